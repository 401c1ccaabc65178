"""TEST INFRASTRUCTURE ONLY: ctypes front end of the reference's own GPU
kernels (oracle/_ref/libref_gpu.so, built by oracle/build_ref.py from
GPU/dyhash/cuckoo.cu of pauline-ly/databases_gpu).

``RefGpuTable`` lays a table out as ``hashAPI::hashAPI`` does (api.cpp:46-74:
4 subtables of nextPrime(size/64) buckets rounded up to even, 16 slots of 8
bytes, zeroed) in torch device memory and runs the reference's insert,
search, delete and resize kernels on it. The tests compare the library with
it; bench.py times its search beside the library's find. One reference table
is live per process (the kernels read a single ``__constant__`` descriptor).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from oracle import build_ref
from oracle import oracle as orc

_lib = None


def available() -> bool:
    """True when libref_gpu.so exists or can be built from staged sources."""
    return os.path.exists(build_ref.GPU_LIB) or build_ref.gpu_staged()


def lib():
    global _lib
    if _lib is not None:
        return _lib
    path = build_ref.build_gpu()
    if path is None:
        raise RuntimeError("reference GPU kernels not staged (oracle/build_ref.py)")
    L = C.CDLL(path)
    vp, u32 = C.c_void_p, C.c_uint32
    sig = {
        "refgpu_geometry": [C.POINTER(C.c_uint32)] * 4,
        "refgpu_set_table": [C.POINTER(C.c_void_p), C.POINTER(C.c_uint32)],
        "refgpu_layout": [C.POINTER(C.c_void_p), C.POINTER(C.c_uint32)],
        "refgpu_insert": [vp, vp, u32, vp, vp, vp],
        "refgpu_search": [vp, vp, u32, vp],
        "refgpu_delete": [vp, u32, vp],
        "refgpu_resize_up": [C.c_int, vp],
        "refgpu_resize_down": [C.c_int, vp],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.restype = C.c_int
        f.argtypes = args
    _lib = L
    return L


def geometry():
    v = [C.c_uint32() for _ in range(4)]
    rc = lib().refgpu_geometry(*[C.byref(x) for x in v])
    assert rc == 0
    return tuple(x.value for x in v)  # blocks, threads, slots per bucket, subtables


def _check(rc, what):
    if rc != 0:
        raise RuntimeError("%s failed (code %d)" % (what, rc))


class RefGpuTable:
    """The reference's table on the GPU, sized by hashAPI(size)."""

    SUBTABLES = 4
    SLOTS = 16

    def __init__(self, size: int, device: int = 0):
        import torch
        self.torch = torch
        self.dev = torch.device("cuda", device)
        nb = orc.subtable_buckets(size, self.SUBTABLES, self.SLOTS)
        self.subtables = [torch.zeros(nb * self.SLOTS, dtype=torch.int64, device=self.dev)
                          for _ in range(self.SUBTABLES)]
        self.rehash = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self._upload()

    def _upload(self):
        ptrs = (C.c_void_p * self.SUBTABLES)(*[s.data_ptr() for s in self.subtables])
        lsz = (C.c_uint32 * self.SUBTABLES)(*[s.numel() for s in self.subtables])
        self.torch.cuda.synchronize(self.dev)
        _check(lib().refgpu_set_table(ptrs, lsz), "refgpu_set_table")

    def layout(self):
        """Buckets per subtable."""
        return [s.numel() // self.SLOTS for s in self.subtables]

    @property
    def capacity(self) -> int:
        return sum(s.numel() for s in self.subtables)

    def _stream(self, stream):
        s = stream if stream is not None else self.torch.cuda.current_stream(self.dev)
        return C.c_void_p(s.cuda_stream)

    def insert(self, keys, vals, stream=None) -> int:
        """cuckoo_insert; returns the kernel's rehash flag (1: an entry was
        dropped at the end of an eviction chain). keys/vals are int32 device
        tensors holding the 32-bit patterns; values must be < 2^31."""
        n = keys.numel()
        iters = self.torch.empty(max(n, 1), dtype=self.torch.int32, device=self.dev)
        self.rehash.zero_()
        _check(lib().refgpu_insert(keys.data_ptr(), vals.data_ptr(), n, self.rehash.data_ptr(),
                                   iters.data_ptr(), self._stream(stream)), "refgpu_insert")
        self.last_iter_counts = iters[:n]
        return int(self.rehash.item())

    def search(self, keys, out=None, stream=None):
        """cuckoo_search into a zeroed int32 tensor (0 = miss or stored 0)."""
        n = keys.numel()
        if out is None:
            out = self.torch.zeros(n, dtype=self.torch.int32, device=self.dev)
        _check(lib().refgpu_search(keys.data_ptr(), out.data_ptr(), n, self._stream(stream)),
               "refgpu_search")
        return out

    def delete(self, keys, stream=None):
        _check(lib().refgpu_delete(keys.data_ptr(), keys.numel(), self._stream(stream)),
               "refgpu_delete")

    def resize_up(self, t: int):
        """GPU_cuckoo_resize_up of subtable t into a zeroed buffer of twice its slots."""
        new = self.torch.zeros(2 * self.subtables[t].numel(), dtype=self.torch.int64,
                               device=self.dev)
        self.torch.cuda.synchronize(self.dev)
        _check(lib().refgpu_resize_up(t, new.data_ptr()), "refgpu_resize_up")
        self.subtables[t] = new

    def resize_down(self, t: int):
        """GPU_cuckoo_resize_down of subtable t (even bucket count only)."""
        nb = self.subtables[t].numel() // self.SLOTS
        if nb % 2:
            raise ValueError("the reference downsize needs an even bucket count (%d)" % nb)
        new = self.torch.zeros(nb // 2 * self.SLOTS, dtype=self.torch.int64, device=self.dev)
        self.torch.cuda.synchronize(self.dev)
        _check(lib().refgpu_resize_down(t, new.data_ptr()), "refgpu_resize_down")
        self.subtables[t] = new

    def pick_up(self) -> int:
        """hashAPI::resize_up's target (api.cpp:115-122), from the oracle's
        restatement pinned to the reference."""
        nb = np.asarray(self.layout(), np.uint32)
        return orc.lib().orc_pick_up_nb(nb, self.SUBTABLES)

    def pick_down(self) -> int:
        nb = np.asarray(self.layout(), np.uint32)
        return orc.lib().orc_pick_down_nb(nb, self.SUBTABLES)

    def export(self):
        """(keys, values) of every occupied slot, as uint32 arrays (a key
        stored twice appears twice)."""
        self.torch.cuda.synchronize(self.dev)
        a = np.concatenate([s.cpu().numpy().view(np.uint64) for s in self.subtables])
        a = a[a != 0]
        return (a >> np.uint64(32)).astype(np.uint32), (a & np.uint64(0xFFFFFFFF)).astype(np.uint32)
