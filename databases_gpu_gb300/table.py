"""Host-side mirror of the reference's DyCuckoo interface over the C ABI.

``DyCuckoo`` is the device-buffer handle (the reference's gpu_lp_* launch
wrappers, GPU/dyhash/cuckoo.h:99-114): keys, values and results are CUDA
tensors. ``hashAPI`` keeps the reference's class surface
(GPU/dyhash/api.h:9-54) with host arrays: hash_insert / hash_search /
hash_delete / resize_up / resize_low and the batch-pool calls.

PyTorch is used only for device memory and streams; every operation is a
call into libdycuckoo.so.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import FLAG_GRAPH, FLAG_NEW_KEYS, FLAG_NO_RESIZE, FLAG_UNIQUE, check

# test_uilt.h:1-5 of the reference
UPPER_BOUND = 0.8
LOWER_BOUND = 0.5
BATCH_NUM = 1000
BATCH_SIZE = 100000
MIN_DOWNSIZE_CAPACITY = int(4 * 1024 * 1024 * 1.2)  # api.cpp:496


def _torch():
    import torch
    return torch


def _ptr(t, what: str, elem_bytes: int | None = None):
    if t is None:
        return None
    torch = _torch()
    if not isinstance(t, torch.Tensor):
        raise TypeError("%s must be a CUDA tensor" % what)
    if not t.is_cuda:
        raise ValueError("%s must live on a CUDA device" % what)
    if not t.is_contiguous():
        raise ValueError("%s must be contiguous" % what)
    if elem_bytes is not None and t.element_size() != elem_bytes:
        raise ValueError("%s must have %d-byte elements, got %s" % (what, elem_bytes, t.dtype))
    return C.c_void_p(t.data_ptr())


def _stream_ptr(stream):
    if stream is None:
        return C.c_void_p(_torch().cuda.current_stream().cuda_stream)
    if isinstance(stream, int):
        return C.c_void_p(stream)
    return C.c_void_p(stream.cuda_stream)


class DyCuckoo:
    """A GB300 DyCuckoo table; all arrays are CUDA tensors.

    size: number of keys to size the table for (the hashAPI(size) argument).
    l2_resident: 2 asks the L2 to keep the buckets (eviction-priority
    hints); 0 (default) and 1 use plain accesses (dyc_config.l2_resident).
    """

    def __init__(self, size: int, key_bytes: int = 4, value_bytes: int | None = None,
                 num_subtables: int = 4, bucket_bytes: int = 128, max_evictions: int = 64,
                 auto_resize: bool = True, upper_load: float = UPPER_BOUND,
                 lower_load: float = LOWER_BOUND,
                 min_downsize_capacity: int = MIN_DOWNSIZE_CAPACITY, device: int = 0,
                 l2_resident: int = 0):
        L = _lib.lib()
        cfg = _lib.DycConfig()
        L.dyc_config_default(C.byref(cfg))
        cfg.key_bytes = key_bytes
        cfg.value_bytes = value_bytes if value_bytes is not None else key_bytes
        cfg.num_subtables = num_subtables
        cfg.bucket_bytes = bucket_bytes
        cfg.max_evictions = max_evictions
        cfg.auto_resize = 1 if auto_resize else 0
        cfg.l2_resident = l2_resident
        cfg.initial_size = int(size)
        cfg.upper_load = upper_load
        cfg.lower_load = lower_load
        cfg.min_downsize_capacity = int(min_downsize_capacity)
        cfg.device = device
        h = C.c_void_p()
        check(L.dyc_create(C.byref(cfg), C.byref(h)), "dyc_create")
        self._h = h
        self.L = L
        self.cfg = cfg
        self.key_bytes = cfg.key_bytes
        self.value_bytes = cfg.value_bytes
        self.device = device

    @classmethod
    def _member(cls, handle, cfg, owner):
        """A non-owning handle on a member table of a DyCuckooSet."""
        t = cls.__new__(cls)
        t._h = handle
        t.L = owner.L
        t.cfg = cfg
        t.key_bytes = cfg.key_bytes
        t.value_bytes = cfg.value_bytes
        t.device = cfg.device
        t._owner = owner  # keeps the owner (set, server, wide table) alive
        return t

    # -- lifetime
    def close(self):
        if getattr(self, "_owner", None) is not None:
            self._h = None  # destroyed with its set
            return
        if getattr(self, "_h", None):
            self.L.dyc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    # -- dtypes
    def key_dtype(self):
        torch = _torch()
        return torch.int32 if self.key_bytes == 4 else torch.int64

    def value_dtype(self):
        torch = _torch()
        return torch.int32 if self.value_bytes == 4 else torch.int64

    # -- batch ops
    def insert(self, keys, values, unique: bool = False, new_keys: bool = False,
               no_resize: bool = False, stream=None) -> dict:
        n = keys.numel()
        if values.numel() != n:
            raise ValueError("keys and values differ in length")
        flags = (FLAG_UNIQUE if unique else 0) | (FLAG_NEW_KEYS if new_keys else 0) | \
            (FLAG_NO_RESIZE if no_resize else 0)
        check(self.L.dyc_insert(self._h, _ptr(keys, "keys", self.key_bytes),
                                _ptr(values, "values", self.value_bytes), n, flags,
                                _stream_ptr(stream)), "dyc_insert")
        return self.stats()

    def find(self, keys, out=None, hit_bits=None, want_hits: bool = True, stream=None):
        torch = _torch()
        n = keys.numel()
        if out is None:
            out = torch.empty(n, dtype=self.value_dtype(), device=keys.device)
        if hit_bits is None and want_hits:
            hit_bits = torch.empty((n + 31) // 32, dtype=torch.int32, device=keys.device)
        check(self.L.dyc_find(self._h, _ptr(keys, "keys", self.key_bytes),
                              _ptr(out, "out", self.value_bytes),
                              _ptr(hit_bits, "hit_bits", 4) if hit_bits is not None else None,
                              n, _stream_ptr(stream)), "dyc_find")
        return out, hit_bits

    def erase(self, keys, erased_bits=None, unique: bool = False, no_resize: bool = False,
              stream=None) -> int:
        n = keys.numel()
        cnt = C.c_uint64(0)
        flags = (FLAG_UNIQUE if unique else 0) | (FLAG_NO_RESIZE if no_resize else 0)
        check(self.L.dyc_erase(self._h, _ptr(keys, "keys", self.key_bytes), n,
                               _ptr(erased_bits, "erased_bits", 4) if erased_bits is not None else None,
                               C.byref(cnt), flags, _stream_ptr(stream)), "dyc_erase")
        return int(cnt.value)

    def apply(self, ops, keys, values, out=None, bits=None, no_resize: bool = False,
              unique: bool = False, stream=None):
        """Mixed batch (dyc_apply): ops is a uint8 tensor of OP_FIND /
        OP_INSERT / OP_ERASE, applied in index order. Returns (out, bits):
        the value each op saw (found / previous / removed, 0 if absent) and
        one bit per op, set when the key was present before the op.
        unique: the caller promises no key repeats in the batch (one probe
        pass per op, DYC_FLAG_UNIQUE)."""
        torch = _torch()
        n = keys.numel()
        if ops.numel() != n or values.numel() != n:
            raise ValueError("ops, keys and values differ in length")
        if ops.dtype != torch.uint8:
            raise TypeError("ops must be uint8")
        if out is None:
            out = torch.empty(n, dtype=self.value_dtype(), device=keys.device)
        if bits is None:
            bits = torch.empty((n + 31) // 32, dtype=torch.int32, device=keys.device)
        check(self.L.dyc_apply(self._h, _ptr(ops, "ops", 1), _ptr(keys, "keys", self.key_bytes),
                               _ptr(values, "values", self.value_bytes),
                               n, _ptr(out, "out", self.value_bytes), _ptr(bits, "bits", 4),
                               (FLAG_NO_RESIZE if no_resize else 0) |
                               (FLAG_UNIQUE if unique else 0), _stream_ptr(stream)),
              "dyc_apply")
        return out, bits

    def resize_up(self, stream=None) -> None:
        check(self.L.dyc_resize_up(self._h, _stream_ptr(stream)), "dyc_resize_up")

    def resize_down(self, stream=None) -> None:
        check(self.L.dyc_resize_down(self._h, _stream_ptr(stream)), "dyc_resize_down")

    # -- introspection
    @property
    def size(self) -> int:
        v = C.c_uint64()
        check(self.L.dyc_size(self._h, C.byref(v)), "dyc_size")
        return int(v.value)

    @property
    def capacity(self) -> int:
        v = C.c_uint64()
        check(self.L.dyc_capacity(self._h, C.byref(v)), "dyc_capacity")
        return int(v.value)

    def layout(self):
        nb = (C.c_uint32 * 6)()
        d = C.c_uint32()
        check(self.L.dyc_layout(self._h, nb, C.byref(d)), "dyc_layout")
        return [int(nb[i]) for i in range(d.value)]

    def stats(self) -> dict:
        s = _lib.DycOpStats()
        check(self.L.dyc_last_stats(self._h, C.byref(s)), "dyc_last_stats")
        return s.as_dict()

    def subtable(self, i: int, with_meta: bool = False):
        """Subtable i on the host: (buckets, slots) raw 64-bit slots for
        4-byte keys, (buckets, slots, 2) for 8-byte keys. 128-byte buckets end
        with a metadata slot, dropped unless with_meta."""
        torch = _torch()
        p = C.c_void_p()
        nbytes = C.c_uint64()
        check(self.L.dyc_subtable(self._h, i, C.byref(p), C.byref(nbytes)), "dyc_subtable")
        torch.cuda.synchronize(self.device)
        host = np.empty(nbytes.value // 8, np.uint64)
        cudart = C.CDLL("libcudart.so.13")
        cudart.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
        rc = cudart.cudaMemcpy(host.ctypes.data, p, nbytes.value, 2)
        if rc != 0:
            raise RuntimeError("cudaMemcpy of subtable failed: %d" % rc)
        slot_words = 1 if self.key_bytes == 4 else 2
        slots = self.cfg.bucket_bytes // (8 * slot_words)
        nb = self.layout()[i]
        a = host.reshape(nb, slots, slot_words) if slot_words == 2 else host.reshape(nb, slots)
        if self.cfg.bucket_bytes == 128 and not with_meta:
            a = a[:, :-1]
        return a

    def export(self, stream=None):
        """All live (key, value) pairs as CUDA tensors, sorted by key."""
        torch = _torch()
        n = self.size
        cap = max(n, 1)
        k = torch.empty(cap, dtype=self.key_dtype(), device="cuda:%d" % self.device)
        v = torch.empty(cap, dtype=self.value_dtype(), device="cuda:%d" % self.device)
        got = C.c_uint64()
        check(self.L.dyc_export(self._h, _ptr(k, "keys"), _ptr(v, "vals"), cap, C.byref(got),
                                _stream_ptr(stream)), "dyc_export")
        m = int(got.value)
        if m > cap:
            raise RuntimeError("export found %d live entries but size is %d" % (m, n))
        k, v = k[:m], v[:m]
        # sort as unsigned
        if self.key_bytes == 4:
            order = torch.argsort(k.to(torch.int64) & 0xFFFFFFFF)
        else:
            kk = k.cpu().numpy().view(np.uint64)
            order = torch.from_numpy(np.argsort(kk, kind="stable")).to(k.device)
        return k[order], v[order]

    # -- snapshot / restore
    def snapshot(self, stream=None) -> np.ndarray:
        """The table as a snapshot buffer (header + raw subtables)."""
        nb = C.c_uint64()
        check(self.L.dyc_snapshot_bytes(self._h, C.byref(nb)), "dyc_snapshot_bytes")
        buf = np.empty(nb.value, np.uint8)
        check(self.L.dyc_snapshot(self._h, buf.ctypes.data, buf.size, _stream_ptr(stream)),
              "dyc_snapshot")
        return buf

    @classmethod
    def restore(cls, buf, device: int = 0) -> "DyCuckoo":
        """A new table from a snapshot buffer (bytes or uint8 array)."""
        a = np.frombuffer(buf, np.uint8) if isinstance(buf, (bytes, bytearray)) else \
            np.ascontiguousarray(buf, np.uint8)
        L = _lib.lib()
        h = C.c_void_p()
        check(L.dyc_restore(a.ctypes.data, a.size, device, C.byref(h)), "dyc_restore")
        hdr = a[:256].view(np.uint32)
        t = cls.__new__(cls)
        cfg = _lib.DycConfig()
        L.dyc_config_default(C.byref(cfg))
        cfg.key_bytes, cfg.value_bytes, cfg.bucket_bytes, cfg.num_subtables = \
            int(hdr[4]), int(hdr[5]), int(hdr[6]), int(hdr[7])
        cfg.max_evictions, cfg.auto_resize = int(hdr[8]), int(hdr[9])
        cfg.device = device
        t._h, t.L, t.cfg = h, L, cfg
        t.key_bytes, t.value_bytes, t.device = cfg.key_bytes, cfg.value_bytes, device
        return t

    def save(self, path: str) -> None:
        self.snapshot().tofile(path)

    @classmethod
    def load(cls, path: str, device: int = 0) -> "DyCuckoo":
        return cls.restore(np.fromfile(path, np.uint8), device)

    # -- host-buffer forms (reference-facing C ABI with host memory)
    def insert_host(self, keys: np.ndarray, values: np.ndarray, flags: int = 0) -> None:
        keys = np.ascontiguousarray(keys)
        values = np.ascontiguousarray(values)
        check(self.L.dyc_insert_host(self._h, keys.ctypes.data, values.ctypes.data,
                                     keys.size, flags), "dyc_insert_host")

    def find_host(self, keys: np.ndarray, out: np.ndarray, hit_bits: np.ndarray | None = None):
        keys = np.ascontiguousarray(keys)
        check(self.L.dyc_find_host(self._h, keys.ctypes.data, out.ctypes.data,
                                   hit_bits.ctypes.data if hit_bits is not None else None,
                                   keys.size), "dyc_find_host")

    def erase_host(self, keys: np.ndarray, erased_bits: np.ndarray | None = None) -> int:
        keys = np.ascontiguousarray(keys)
        cnt = C.c_uint64()
        check(self.L.dyc_erase_host(self._h, keys.ctypes.data, keys.size,
                                    erased_bits.ctypes.data if erased_bits is not None else None,
                                    C.byref(cnt)), "dyc_erase_host")
        return int(cnt.value)


class DyCuckooSet:
    """Many independent DyCuckoo tables served together (dyc_set_*): one
    launch sequence per mixed batch for the whole set.

    sizes: per-table key counts to size for; num_subtables: optional
    per-table subtable counts; device_upsize: 0 applies a round's upsize
    policy on the device from upsize targets allocated ahead, 1 on the host
    between the round's phases (dyc_config.device_upsize). Other arguments
    as for DyCuckoo (shared)."""

    def __init__(self, sizes, key_bytes: int = 4, value_bytes: int | None = None,
                 num_subtables=None, bucket_bytes: int = 128, max_evictions: int = 64,
                 auto_resize: bool = True, upper_load: float = UPPER_BOUND,
                 lower_load: float = LOWER_BOUND,
                 min_downsize_capacity: int = MIN_DOWNSIZE_CAPACITY, device: int = 0,
                 default_subtables: int = 4, l2_resident: int = 0, device_upsize: int = 0):
        L = _lib.lib()
        cfg = _lib.DycConfig()
        L.dyc_config_default(C.byref(cfg))
        cfg.l2_resident = l2_resident
        cfg.device_upsize = device_upsize
        cfg.key_bytes = key_bytes
        cfg.value_bytes = value_bytes if value_bytes is not None else key_bytes
        cfg.num_subtables = default_subtables
        cfg.bucket_bytes = bucket_bytes
        cfg.max_evictions = max_evictions
        cfg.auto_resize = 1 if auto_resize else 0
        cfg.upper_load = upper_load
        cfg.lower_load = lower_load
        cfg.min_downsize_capacity = int(min_downsize_capacity)
        cfg.device = device
        sz = np.ascontiguousarray(sizes, dtype=np.uint64)
        ns = None if num_subtables is None else np.ascontiguousarray(num_subtables, np.uint32)
        h = C.c_void_p()
        check(L.dyc_set_create(C.byref(cfg), sz.size, sz.ctypes.data,
                               ns.ctypes.data if ns is not None else None, C.byref(h)),
              "dyc_set_create")
        self._h = h
        self.L = L
        self.cfg = cfg
        self.ntables = int(sz.size)
        self.key_bytes = cfg.key_bytes
        self.value_bytes = cfg.value_bytes
        self.device = device

    def close(self):
        if getattr(self, "_h", None):
            self.L.dyc_set_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def configure(self, blocks_per_sm: int = 0, max_evictions=None) -> None:
        """Launch cap of the set kernels and per-table eviction bounds."""
        ev = None if max_evictions is None else np.ascontiguousarray(max_evictions, np.uint32)
        if ev is not None and ev.size != self.ntables:
            raise ValueError("one eviction bound per table")
        check(self.L.dyc_set_configure(self._h, int(blocks_per_sm),
                                       ev.ctypes.data if ev is not None else None),
              "dyc_set_configure")

    def table(self, i: int) -> DyCuckoo:
        h = C.c_void_p()
        check(self.L.dyc_set_table(self._h, i, C.byref(h)), "dyc_set_table")
        cfg = _lib.DycConfig()
        C.memmove(C.byref(cfg), C.byref(self.cfg), C.sizeof(cfg))
        return DyCuckoo._member(h, cfg, self)

    def sizes(self):
        s = np.empty(self.ntables, np.uint64)
        c = np.empty(self.ntables, np.uint64)
        check(self.L.dyc_set_sizes(self._h, s.ctypes.data, c.ctypes.data), "dyc_set_sizes")
        return s, c

    def stats(self) -> dict:
        st = _lib.DycOpStats()
        check(self.L.dyc_set_last_stats(self._h, C.byref(st)), "dyc_set_last_stats")
        return st.as_dict()

    def spare_bytes(self) -> int:
        """Device bytes held beside the members' subtables (upsize targets
        allocated ahead, replaced subtables not yet freed)."""
        b = C.c_uint64()
        check(self.L.dyc_set_spare_bytes(self._h, C.byref(b)), "dyc_set_spare_bytes")
        return int(b.value)

    def spare_cache(self, max_bytes: int) -> None:
        """Bound the replaced subtables kept for reuse as upsize targets
        (dyc_set_spare_cache; 0 keeps none)."""
        check(self.L.dyc_set_spare_cache(self._h, int(max_bytes)), "dyc_set_spare_cache")

    def apply(self, offsets, ops, keys, values, out=None, bits=None, h_offsets=None,
              each: bool = False, graph: bool = False, no_resize: bool = False, stream=None):
        """Mixed batch: ops of table t are [offsets[t], offsets[t+1]) of the
        op / key / value tensors. offsets: uint32 CUDA tensor of ntables+1
        (h_offsets: its host copy, computed if omitted). each: one dyc_apply
        per table instead (the per-table launch path). Returns (out, bits)."""
        torch = _torch()
        n = keys.numel()
        if h_offsets is None:
            h_offsets = offsets.cpu().numpy()
        h_offsets = np.ascontiguousarray(np.asarray(h_offsets).view(np.uint32)
                                         if np.asarray(h_offsets).dtype == np.int32
                                         else np.asarray(h_offsets, dtype=np.uint32))
        if h_offsets.size != self.ntables + 1 or int(h_offsets[-1]) != n:
            raise ValueError("offsets must have ntables+1 entries ending at the op count")
        if out is None:
            out = torch.empty(n, dtype=torch.int32 if self.value_bytes == 4 else torch.int64,
                              device=keys.device)
        if bits is None:
            bits = torch.empty((n + 31) // 32, dtype=torch.int32, device=keys.device)
        flags = (FLAG_NO_RESIZE if no_resize else 0) | (FLAG_GRAPH if graph else 0)
        fn = self.L.dyc_set_apply_each if each else self.L.dyc_set_apply
        check(fn(self._h, _ptr(offsets, "offsets", 4), h_offsets.ctypes.data,
                 _ptr(ops, "ops", 1), _ptr(keys, "keys", self.key_bytes),
                 _ptr(values, "values", self.value_bytes), _ptr(out, "out", self.value_bytes),
                 _ptr(bits, "bits", 4), flags, _stream_ptr(stream)),
              "dyc_set_apply_each" if each else "dyc_set_apply")
        return out, bits


class DyCuckooWide:
    """Table with values of value_bytes (a multiple of 4) per key (dyc_wide_*).
    Keys: CUDA tensor of int32/int64; values: CUDA tensor of n * value_bytes
    bytes, e.g. shape (n, value_bytes // 4) int32."""

    def __init__(self, size: int, value_bytes: int, key_bytes: int = 4, num_subtables: int = 4,
                 bucket_bytes: int = 128, max_evictions: int = 64, auto_resize: bool = True,
                 upper_load: float = UPPER_BOUND, lower_load: float = LOWER_BOUND,
                 min_downsize_capacity: int = MIN_DOWNSIZE_CAPACITY, device: int = 0):
        L = _lib.lib()
        cfg = _lib.DycConfig()
        L.dyc_config_default(C.byref(cfg))
        cfg.key_bytes, cfg.value_bytes = key_bytes, 4
        cfg.num_subtables, cfg.bucket_bytes = num_subtables, bucket_bytes
        cfg.max_evictions, cfg.auto_resize = max_evictions, 1 if auto_resize else 0
        cfg.initial_size = int(size)
        cfg.upper_load, cfg.lower_load = upper_load, lower_load
        cfg.min_downsize_capacity = int(min_downsize_capacity)
        cfg.device = device
        h = C.c_void_p()
        check(L.dyc_wide_create(C.byref(cfg), value_bytes, C.byref(h)), "dyc_wide_create")
        self._h, self.L, self.cfg = h, L, cfg
        self.key_bytes, self.value_bytes, self.device = key_bytes, value_bytes, device

    def close(self):
        if getattr(self, "_h", None):
            self.L.dyc_wide_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _vals(self, v, n, what):
        if v.numel() * v.element_size() != n * self.value_bytes:
            raise ValueError("%s must hold %d bytes per key" % (what, self.value_bytes))
        return _ptr(v, what)

    def insert(self, keys, values, unique: bool = False, no_resize: bool = False, stream=None):
        n = keys.numel()
        flags = (FLAG_UNIQUE if unique else 0) | (FLAG_NO_RESIZE if no_resize else 0)
        check(self.L.dyc_wide_insert(self._h, _ptr(keys, "keys", self.key_bytes),
                                     self._vals(values, n, "values"), n, flags,
                                     _stream_ptr(stream)), "dyc_wide_insert")
        return self.stats()

    def find(self, keys, stream=None):
        torch = _torch()
        n = keys.numel()
        out = torch.empty((n, self.value_bytes // 4), dtype=torch.int32, device=keys.device)
        bits = torch.empty((n + 31) // 32, dtype=torch.int32, device=keys.device)
        check(self.L.dyc_wide_find(self._h, _ptr(keys, "keys", self.key_bytes), _ptr(out, "out"),
                                   _ptr(bits, "bits", 4), n, _stream_ptr(stream)), "dyc_wide_find")
        return out, bits

    def erase(self, keys, no_resize: bool = False, stream=None):
        """(count removed, removed values (zeros where nothing was removed), erased bits)"""
        torch = _torch()
        n = keys.numel()
        out = torch.empty((n, self.value_bytes // 4), dtype=torch.int32, device=keys.device)
        bits = torch.empty((n + 31) // 32, dtype=torch.int32, device=keys.device)
        cnt = C.c_uint64()
        check(self.L.dyc_wide_erase(self._h, _ptr(keys, "keys", self.key_bytes), n,
                                    _ptr(out, "out"), _ptr(bits, "bits", 4), C.byref(cnt),
                                    FLAG_NO_RESIZE if no_resize else 0, _stream_ptr(stream)),
              "dyc_wide_erase")
        return int(cnt.value), out, bits

    def table(self) -> DyCuckoo:
        h = C.c_void_p()
        check(self.L.dyc_wide_table(self._h, C.byref(h)), "dyc_wide_table")
        cfg = _lib.DycConfig()
        C.memmove(C.byref(cfg), C.byref(self.cfg), C.sizeof(cfg))
        return DyCuckoo._member(h, cfg, self)

    @property
    def size(self) -> int:
        return self.table().size

    def stats(self) -> dict:
        st = _lib.DycOpStats()
        check(self.L.dyc_wide_last_stats(self._h, C.byref(st)), "dyc_wide_last_stats")
        return st.as_dict()

    def export(self, stream=None):
        """(keys, values (n, value_bytes // 4) int32) of every live entry, sorted by key."""
        torch = _torch()
        n = self.size
        cap = max(n, 1)
        dev = "cuda:%d" % self.device
        k = torch.empty(cap, dtype=torch.int32 if self.key_bytes == 4 else torch.int64, device=dev)
        v = torch.empty((cap, self.value_bytes // 4), dtype=torch.int32, device=dev)
        got = C.c_uint64()
        check(self.L.dyc_wide_export(self._h, _ptr(k, "keys"), _ptr(v, "vals"), cap,
                                     C.byref(got), _stream_ptr(stream)), "dyc_wide_export")
        m = int(got.value)
        k, v = k[:m], v[:m]
        kk = k.cpu().numpy().view(np.uint32 if self.key_bytes == 4 else np.uint64)
        order = torch.from_numpy(np.argsort(kk, kind="stable")).to(k.device)
        return k[order], v[order]


class DyCuckooServer:
    """Request server over per-tenant tables (dyc_server_*): submit mixed-op
    requests in host memory from any thread, wait for their results.

    sizes: per-tenant key counts to size for; hbm_cap_bytes: admission cap
    (0: none); coalesce: continuous batching (False: one request per step)."""

    def __init__(self, sizes, key_bytes: int = 8, value_bytes: int = 4,
                 hbm_cap_bytes: int = 0, max_step_ops: int = 1 << 22, coalesce: bool = True,
                 bucket_bytes: int = 128, max_evictions: int = 64, auto_resize: bool = True,
                 upper_load: float = UPPER_BOUND, lower_load: float = LOWER_BOUND,
                 min_downsize_capacity: int = MIN_DOWNSIZE_CAPACITY, device: int = 0):
        import threading
        L = _lib.lib()
        cfg = _lib.DycConfig()
        L.dyc_config_default(C.byref(cfg))
        cfg.key_bytes, cfg.value_bytes = key_bytes, value_bytes
        cfg.bucket_bytes, cfg.max_evictions = bucket_bytes, max_evictions
        cfg.auto_resize = 1 if auto_resize else 0
        cfg.upper_load, cfg.lower_load = upper_load, lower_load
        cfg.min_downsize_capacity = int(min_downsize_capacity)
        cfg.device = device
        sc = _lib.DycServerConfig()
        L.dyc_server_config_default(C.byref(sc))
        sc.hbm_cap_bytes = int(hbm_cap_bytes)
        sc.max_step_ops = int(max_step_ops)
        sc.coalesce = 1 if coalesce else 0
        sz = np.ascontiguousarray(sizes, dtype=np.uint64)
        h = C.c_void_p()
        check(L.dyc_server_create(C.byref(cfg), sz.size, sz.ctypes.data, C.byref(sc),
                                  C.byref(h)), "dyc_server_create")
        self._h, self.L, self.cfg = h, L, cfg
        self.ntenants = int(sz.size)
        self.key_bytes, self.value_bytes = key_bytes, value_bytes
        self._keep = {}  # ticket -> arrays the server reads / writes
        self._lock = threading.Lock()

    def close(self):
        if getattr(self, "_h", None):
            self.L.dyc_server_destroy(self._h)
            self._h = None
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, tenant: int, ops: np.ndarray, keys: np.ndarray, vals: np.ndarray) -> int:
        """Queue a request; returns its ticket. Results come from wait()."""
        ops = np.ascontiguousarray(ops, np.uint8)
        keys = np.ascontiguousarray(keys)
        vals = np.ascontiguousarray(vals)
        n = ops.size
        if keys.itemsize != self.key_bytes or vals.itemsize != self.value_bytes:
            raise ValueError("key / value widths do not match the server")
        out = np.empty(n, np.uint32 if self.value_bytes == 4 else np.uint64)
        bits = np.empty((n + 31) // 32, np.uint32)
        t = C.c_uint64()
        check(self.L.dyc_server_submit(self._h, tenant, ops.ctypes.data, keys.ctypes.data,
                                       vals.ctypes.data, n, out.ctypes.data, bits.ctypes.data,
                                       C.byref(t)), "dyc_server_submit")
        with self._lock:
            self._keep[t.value] = (ops, keys, vals, out, bits, n)
        return int(t.value)

    def wait(self, ticket: int, timeout_ms: int = -1):
        """(status, values, hit bits as bool array, latency in ns)."""
        st = C.c_int()
        lat = C.c_uint64()
        check(self.L.dyc_server_wait(self._h, ticket, timeout_ms, C.byref(st), C.byref(lat)),
              "dyc_server_wait")
        with self._lock:
            ops, keys, vals, out, bits, n = self._keep.pop(ticket)
        return int(st.value), out, unpack_bits(bits, n), int(lat.value)

    def stats(self) -> dict:
        s = _lib.DycServerStats()
        check(self.L.dyc_server_stats_get(self._h, C.byref(s)), "dyc_server_stats_get")
        return s.as_dict()

    def table(self, i: int) -> DyCuckoo:
        """Tenant i's table (use only while nothing is queued or running)."""
        hs = C.c_void_p()
        check(self.L.dyc_server_set(self._h, C.byref(hs)), "dyc_server_set")
        h = C.c_void_p()
        check(self.L.dyc_set_table(hs, i, C.byref(h)), "dyc_set_table")
        cfg = _lib.DycConfig()
        C.memmove(C.byref(cfg), C.byref(self.cfg), C.sizeof(cfg))
        return DyCuckoo._member(h, cfg, self)


def pool_reserve(nbytes: int, device: int = 0) -> None:
    """Map nbytes of device memory into the library's allocation pool now
    (dyc_pool_reserve), so later resizes on `device` reuse it."""
    L = _lib.lib()
    check(L.dyc_pool_reserve(device, int(nbytes)), "dyc_pool_reserve")


def unpack_bits(bits, n: int) -> np.ndarray:
    """Hit / erased bit words (ceil(n/32) uint32) -> bool array of n."""
    if hasattr(bits, "cpu"):
        bits = bits.cpu().numpy()
    w = np.asarray(bits).view(np.uint32)
    b = np.unpackbits(w.view(np.uint8), bitorder="little")
    return b[:n].astype(bool)


class hashAPI:  # noqa: N801 -- the reference's class name
    """The reference's hashAPI (GPU/dyhash/api.h:9-54, api.cpp) on GB300.

    Host arrays in, host arrays out, like the reference. Differences, all
    deliberate: the 4 GiB the reference's constructor gives its CNMeM pool
    (api.cpp:37-40) are mapped into the library's stream-ordered pool
    (dyc_pool_reserve); no leaked buffers; any number of live tables; sizes
    are exact counts (the reference's num_size counts nominal batch sizes,
    api.cpp:371, :490); insert is an upsert and no entry is ever dropped (the
    reference drops entries at the end of long eviction chains,
    cuckoo.cu:422-431).
    """

    POOL_BYTES = 4 << 30

    def __init__(self, size: int, **cfg):
        cfg.setdefault("auto_resize", False)  # hash_insert has the check compiled out (api.cpp:185)
        self.t = DyCuckoo(int(size), **cfg)
        pool_reserve(self.POOL_BYTES, device=self.t.device)
        self._pool_k = None
        self._pool_v = None
        self.batch_num_to_op = 0
        self.batch_del_num_to_op = 0
        self.batch_search_num_to_op = 0

    def close(self):
        self.t.close()

    @property
    def table_size(self) -> int:
        return self.t.capacity

    @property
    def num_size(self) -> int:
        return self.t.size

    # api.cpp:184-265
    def hash_insert(self, k: np.ndarray, v: np.ndarray, size: int) -> None:
        kd = np.uint32 if self.t.key_bytes == 4 else np.uint64
        vd = np.uint32 if self.t.value_bytes == 4 else np.uint64
        self.t.insert_host(np.ascontiguousarray(k[:size], kd), np.ascontiguousarray(v[:size], vd))

    # api.cpp:267-285: ans[i] = value, 0 on a miss
    def hash_search(self, k: np.ndarray, ans: np.ndarray, size: int) -> None:
        kd = np.uint32 if self.t.key_bytes == 4 else np.uint64
        vd = np.uint32 if self.t.value_bytes == 4 else np.uint64
        out = np.empty(size, vd)
        self.t.find_host(np.ascontiguousarray(k[:size], kd), out)
        ans[:size] = out

    # api.cpp:289-303: the reference returns zeros in ans; this returns the
    # number of keys removed as well
    def hash_delete(self, k: np.ndarray, ans: np.ndarray, size: int) -> int:
        kd = np.uint32 if self.t.key_bytes == 4 else np.uint64
        n = self.t.erase_host(np.ascontiguousarray(k[:size], kd))
        ans[:size] = 0
        return n

    # api.cpp:112-141, :143-173
    def resize_up(self) -> None:
        self.t.resize_up()

    def resize_low(self) -> None:
        self.t.resize_down()

    # ---- batch pool (api.cpp:309-506)
    def set_data_to_gpu(self, key: np.ndarray, value: np.ndarray, size: int) -> bool:
        torch = _torch()
        if size > (1 << 30) // 8:
            raise ValueError("set data error size of kv out of 2G")
        kd = torch.int32 if self.t.key_bytes == 4 else torch.int64
        vd = torch.int32 if self.t.value_bytes == 4 else torch.int64
        dev = "cuda:%d" % self.t.device
        self._pool_k = torch.from_numpy(np.ascontiguousarray(key[:size]).view(
            np.int32 if kd == torch.int32 else np.int64)).to(dev)
        self._pool_v = torch.from_numpy(np.ascontiguousarray(value[:size]).view(
            np.int32 if vd == torch.int32 else np.int64)).to(dev)
        self._check = torch.zeros(BATCH_SIZE, dtype=vd, device=dev)
        return True

    def batch_reset(self) -> None:
        self.batch_num_to_op = 0
        self.batch_del_num_to_op = 0
        self.batch_search_num_to_op = 0

    def _batch(self, i: int):
        lo = i * BATCH_SIZE
        return self._pool_k[lo:lo + BATCH_SIZE], self._pool_v[lo:lo + BATCH_SIZE]

    def hash_insert_batch(self) -> None:
        if self.batch_num_to_op >= BATCH_NUM:
            raise IndexError("batch_num_to_op >= BATCH_NUM")
        k, v = self._batch(self.batch_num_to_op)
        self._insert_with_policy(k, v)
        self.batch_num_to_op += 1

    def hash_search_batch(self) -> None:
        if self.batch_search_num_to_op >= BATCH_NUM:
            raise IndexError("batch_search_num_to_op >= BATCH_NUM")
        k, _ = self._batch(self.batch_search_num_to_op)
        self.t.find(k, out=self._check[:k.numel()], want_hits=False)
        self.batch_search_num_to_op += 1

    def hash_delete_batch(self) -> None:
        if self.batch_del_num_to_op >= BATCH_NUM:
            raise IndexError("batch_del_num_to_op >= BATCH_NUM")
        k, _ = self._batch(self.batch_del_num_to_op)
        self._erase_with_policy(k)
        self.batch_del_num_to_op += 1

    def _insert_with_policy(self, k, v):
        # projected-size upsize loop of hash_insert_batch (api.cpp:359-369)
        while self.t.size + k.numel() > UPPER_BOUND * self.t.capacity:
            self.t.resize_up()
        self.t.insert(k, v, no_resize=True)

    def _erase_with_policy(self, k):
        self.t.erase(k, no_resize=True)
        # one downsize after a delete batch (api.cpp:494-505)
        if self.t.size < LOWER_BOUND * self.t.capacity and \
                self.t.capacity > MIN_DOWNSIZE_CAPACITY:
            self.t.resize_down()
