"""GB300-native DyCuckoo dynamic hash table (the GPU/dyhash hot path of
pauline-ly/databases_gpu), as sm_103a CUDA kernels behind a C ABI
(include/dycuckoo.h, libdycuckoo.so)."""
from ._lib import DycError, lib, library_path  # noqa: F401
from .table import DyCuckoo, DyCuckooServer, DyCuckooSet, hashAPI, unpack_bits  # noqa: F401

__all__ = ["DyCuckoo", "hashAPI", "unpack_bits", "DycError", "lib", "library_path"]
