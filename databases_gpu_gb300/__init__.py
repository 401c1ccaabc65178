"""GB300-native DyCuckoo dynamic hash table (the GPU/dyhash hot path of
pauline-ly/databases_gpu), as sm_103a CUDA kernels behind a C ABI
(include/dycuckoo.h, libdycuckoo.so)."""
from ._lib import DycError, lib, library_path  # noqa: F401
from .table import (DyCuckoo, DyCuckooServer, DyCuckooSet, DyCuckooWide, hashAPI,  # noqa: F401
                    pool_reserve, unpack_bits)

__all__ = ["DyCuckoo", "DyCuckooSet", "DyCuckooServer", "DyCuckooWide", "hashAPI", "pool_reserve",
           "unpack_bits",
           "DycError", "lib", "library_path"]
