"""ctypes binding of libdycuckoo.so (the C ABI in include/dycuckoo.h).

Loading builds the library in-tree when it is missing or stale and nvcc is
available; otherwise it raises. There is no CPU fallback: every table
operation runs the CUDA kernels of the library.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

DYC_OK, DYC_ENOMEM, DYC_EINVAL, DYC_EOVERFLOW, DYC_ETIMEOUT, DYC_ECUDA, DYC_ENOTSUP = range(7)
FLAG_UNIQUE, FLAG_NEW_KEYS, FLAG_NO_RESIZE, FLAG_GRAPH = 1, 2, 4, 8
OP_FIND, OP_INSERT, OP_ERASE = 0, 1, 2  # dyc_apply op codes


class DycConfig(C.Structure):
    _fields_ = [
        ("key_bytes", C.c_uint32),
        ("value_bytes", C.c_uint32),
        ("num_subtables", C.c_uint32),
        ("bucket_bytes", C.c_uint32),
        ("max_evictions", C.c_uint32),
        ("auto_resize", C.c_uint32),
        ("initial_size", C.c_uint64),
        ("upper_load", C.c_double),
        ("lower_load", C.c_double),
        ("min_downsize_capacity", C.c_uint64),
        ("device", C.c_int32),
        ("l2_resident", C.c_uint32),
        ("device_upsize", C.c_uint32),
        ("reserved", C.c_uint32 * 5),
    ]


class DycOpStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in (
        "inserted", "updated", "erased", "rejected", "superseded", "evict_steps",
        "overflowed", "resizes_up", "resizes_down", "split_phases", "held")]

    def as_dict(self):
        return {n: int(getattr(self, n)) for n, _ in self._fields_}


class DycServerConfig(C.Structure):
    _fields_ = [("hbm_cap_bytes", C.c_uint64), ("max_step_ops", C.c_uint64),
                ("coalesce", C.c_uint32), ("pad0", C.c_uint32),
                ("pool_reserve_bytes", C.c_uint64), ("reserved", C.c_uint32 * 4)]


class DycServerStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in (
        "requests", "ops", "steps", "deferred", "rejected", "max_step_ops", "device_bytes")] + \
        [("busy_seconds", C.c_double), ("resizes_up", C.c_uint64), ("resizes_down", C.c_uint64),
         ("resize_step_seconds", C.c_double), ("assemble_seconds", C.c_double),
         ("exec_idle_seconds", C.c_double), ("upload_late_steps", C.c_uint64),
         ("split_steps", C.c_uint64)]

    def as_dict(self):
        return {n: (float if t is C.c_double else int)(getattr(self, n))
                for n, t in self._fields_}


EXPORTS = [
    "dyc_config_default", "dyc_create", "dyc_destroy", "dyc_insert", "dyc_find", "dyc_erase",
    "dyc_resize_up", "dyc_resize_down", "dyc_size", "dyc_capacity", "dyc_layout",
    "dyc_subtable", "dyc_export", "dyc_last_stats", "dyc_insert_host", "dyc_find_host",
    "dyc_erase_host", "dyc_status_string", "dyc_last_error", "dyc_erase_noalloc", "dyc_apply",
    "dyc_pool_reserve",
    "dyc_set_create", "dyc_set_destroy", "dyc_set_table", "dyc_set_sizes", "dyc_set_apply",
    "dyc_set_apply_each", "dyc_set_last_stats", "dyc_set_configure", "dyc_set_spare_bytes",
    "dyc_set_spare_cache",
    "dyc_server_config_default", "dyc_server_create", "dyc_server_destroy", "dyc_server_submit",
    "dyc_server_wait", "dyc_server_stats_get", "dyc_server_set",
    "dyc_snapshot_bytes", "dyc_snapshot", "dyc_restore",
    "dyc_wide_create", "dyc_wide_destroy", "dyc_wide_insert", "dyc_wide_find", "dyc_wide_erase",
    "dyc_wide_export", "dyc_wide_table", "dyc_wide_last_stats", "dyc_debug_inject",
    "dyc_debug_alloc_count",
]
INJECT_RESET, INJECT_POOL_ALLOC, INJECT_WAIT_TRIES, INJECT_CHUNK_OPS = 0, 1, 2, 3  # dyc_debug_inject kinds

_lock = threading.Lock()
_lib = None


def _declare(L):
    vp, u64, u32 = C.c_void_p, C.c_uint64, C.c_uint32
    st = C.c_int
    T = C.c_void_p
    sig = {
        "dyc_config_default": (None, [C.POINTER(DycConfig)]),
        "dyc_create": (st, [C.POINTER(DycConfig), C.POINTER(C.c_void_p)]),
        "dyc_destroy": (st, [T]),
        "dyc_pool_reserve": (st, [C.c_int32, u64]),
        "dyc_insert": (st, [T, vp, vp, u64, u32, vp]),
        "dyc_find": (st, [T, vp, vp, vp, u64, vp]),
        "dyc_erase": (st, [T, vp, u64, vp, C.POINTER(u64), u32, vp]),
        "dyc_resize_up": (st, [T, vp]),
        "dyc_resize_down": (st, [T, vp]),
        "dyc_size": (st, [T, C.POINTER(u64)]),
        "dyc_capacity": (st, [T, C.POINTER(u64)]),
        "dyc_layout": (st, [T, C.POINTER(u32), C.POINTER(u32)]),
        "dyc_subtable": (st, [T, u32, C.POINTER(vp), C.POINTER(u64)]),
        "dyc_export": (st, [T, vp, vp, u64, C.POINTER(u64), vp]),
        "dyc_last_stats": (st, [T, C.POINTER(DycOpStats)]),
        "dyc_insert_host": (st, [T, vp, vp, u64, u32]),
        "dyc_find_host": (st, [T, vp, vp, vp, u64]),
        "dyc_erase_host": (st, [T, vp, u64, vp, C.POINTER(u64)]),
        "dyc_erase_noalloc": (st, [T, vp, u64, vp, C.POINTER(u64), u32, vp]),
        "dyc_apply": (st, [T, vp, vp, vp, u64, vp, vp, u32, vp]),
        "dyc_set_create": (st, [C.POINTER(DycConfig), u32, vp, vp, C.POINTER(C.c_void_p)]),
        "dyc_set_destroy": (st, [T]),
        "dyc_set_table": (st, [T, u32, C.POINTER(C.c_void_p)]),
        "dyc_set_sizes": (st, [T, vp, vp]),
        "dyc_set_spare_bytes": (st, [T, C.POINTER(C.c_uint64)]),
        "dyc_set_spare_cache": (st, [T, u64]),
        "dyc_set_apply": (st, [T, vp, vp, vp, vp, vp, vp, vp, u32, vp]),
        "dyc_set_apply_each": (st, [T, vp, vp, vp, vp, vp, vp, vp, u32, vp]),
        "dyc_set_last_stats": (st, [T, C.POINTER(DycOpStats)]),
        "dyc_set_configure": (st, [T, u32, vp]),
        "dyc_server_config_default": (None, [C.POINTER(DycServerConfig)]),
        "dyc_server_create": (st, [C.POINTER(DycConfig), u32, vp, C.POINTER(DycServerConfig),
                                   C.POINTER(C.c_void_p)]),
        "dyc_server_destroy": (st, [T]),
        "dyc_server_submit": (st, [T, u32, vp, vp, vp, u64, vp, vp, C.POINTER(u64)]),
        "dyc_server_wait": (st, [T, u64, C.c_int64, C.POINTER(st), C.POINTER(u64)]),
        "dyc_server_stats_get": (st, [T, C.POINTER(DycServerStats)]),
        "dyc_server_set": (st, [T, C.POINTER(C.c_void_p)]),
        "dyc_snapshot_bytes": (st, [T, C.POINTER(u64)]),
        "dyc_snapshot": (st, [T, vp, u64, vp]),
        "dyc_restore": (st, [vp, u64, C.c_int32, C.POINTER(C.c_void_p)]),
        "dyc_wide_create": (st, [C.POINTER(DycConfig), u32, C.POINTER(C.c_void_p)]),
        "dyc_wide_destroy": (st, [T]),
        "dyc_wide_insert": (st, [T, vp, vp, u64, u32, vp]),
        "dyc_wide_find": (st, [T, vp, vp, vp, u64, vp]),
        "dyc_wide_erase": (st, [T, vp, u64, vp, vp, C.POINTER(u64), u32, vp]),
        "dyc_wide_export": (st, [T, vp, vp, u64, C.POINTER(u64), vp]),
        "dyc_wide_table": (st, [T, C.POINTER(C.c_void_p)]),
        "dyc_wide_last_stats": (st, [T, C.POINTER(DycOpStats)]),
        "dyc_debug_inject": (st, [u32, u64]),
        "dyc_debug_alloc_count": (st, [C.POINTER(u64)]),
        "dyc_status_string": (C.c_char_p, [st]),
        "dyc_last_error": (C.c_char_p, []),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args


def lib(path: str | None = None):
    """Load (building first if needed) and return the C library.

    DYCUCKOO_LIB names a prebuilt libdycuckoo.so to load instead of the
    in-tree one (for example a build with other launch parameters)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or os.environ.get("DYCUCKOO_LIB") or _build.LIB
        if p == _build.LIB and (not os.path.exists(p) or not _build.up_to_date(p)):
            _build.build()
        L = C.CDLL(p)
        _declare(L)
        _lib = L
        return L


def library_path() -> str:
    return os.environ.get("DYCUCKOO_LIB") or _build.LIB


class DycError(RuntimeError):
    def __init__(self, status: int, where: str):
        L = lib()
        msg = L.dyc_last_error().decode(errors="replace")
        name = L.dyc_status_string(status).decode()
        super().__init__("%s failed: %s (%d): %s" % (where, name, status, msg))
        self.status = status


def check(status: int, where: str) -> None:
    if status != DYC_OK:
        raise DycError(status, where)
