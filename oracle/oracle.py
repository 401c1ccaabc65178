"""TEST INFRASTRUCTURE ONLY: ctypes front end of the oracle (dyc_oracle.c).

The oracle restates the reference's DyCuckoo algorithm (GPU/dyhash) on the
CPU. tests/, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py`` use
it as the checker and as the timed CPU baseline; the product package never
imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "dyc_oracle.c")
LIB = os.path.join(HERE, "liborc.so")

OP_FIND, OP_INSERT, OP_ERASE = 0, 1, 2

_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")


def build(force: bool = False) -> str:
    """Compile dyc_oracle.c into liborc.so next to it (gcc, no GPU needed)."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(
        os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "dyc_oracle.h"))
    ):
        tmp = LIB + ".tmp%d" % os.getpid()
        subprocess.check_call(
            ["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-pthread", "-Wall",
             "-o", tmp, SRC])
        os.replace(tmp, LIB)
    return LIB


class _MT(C.Structure):
    _fields_ = [("mt", C.c_uint32 * 624), ("mti", C.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is not None:
        return _lib
    build()
    L = C.CDLL(LIB)
    P = C.POINTER(_MT)
    sig = {
        "orc_mt_seed": (None, [P, C.c_uint32]),
        "orc_mt_u32": (C.c_uint32, [P]),
        "orc_mt_u31": (C.c_uint32, [P]),
        "orc_mt_real1": (C.c_double, [P]),
        "orc_mt_fill_u32": (None, [P, _u32p, C.c_uint64]),
        "orc_shuffle": (None, [P, C.c_uint32, _u32p]),
        "orc_gen_unique_ref": (C.c_int, [P, _u32p, C.c_uint32, C.c_uint32]),
        "orc_gen_unique_full": (C.c_int, [P, _u32p, C.c_uint32]),
        "orc_gen_queries": (None, [P, C.c_uint32, C.c_float, _u32p, _u32p]),
        "orc_hash1": (C.c_uint32, [C.c_uint32]),
        "orc_hash2": (C.c_uint32, [C.c_uint32]),
        "orc_hash3": (C.c_uint32, [C.c_uint32]),
        "orc_hash4": (C.c_uint32, [C.c_uint32]),
        "orc_hash5": (C.c_uint32, [C.c_uint32]),
        "orc_fold64": (C.c_uint32, [C.c_uint64]),
        "orc_bucket_of": (C.c_uint32, [C.c_uint32, C.c_uint32, C.c_uint32]),
        "orc_choose_hash": (C.c_uint32, [C.c_uint32, C.c_uint32]),
        "orc_pos1": (C.c_uint32, [C.c_uint32, C.c_uint32]),
        "orc_pos2": (C.c_uint32, [C.c_uint32, C.c_uint32]),
        "orc_hash_batch": (None, [_u32p, C.c_uint64, C.c_uint32, _u32p, _u32p, _u32p,
                                  _u32p, _u32p]),
        "orc_is_prime": (C.c_int, [C.c_int32]),
        "orc_next_prime": (C.c_uint32, [C.c_uint32]),
        "orc_subtable_buckets": (C.c_uint32, [C.c_uint64, C.c_uint32, C.c_uint32]),
        "orc_pick_up_nb": (C.c_int, [_u32p, C.c_uint32]),
        "orc_pick_down_nb": (C.c_int, [_u32p, C.c_uint32]),
        "orc_ck_new": (C.c_void_p, [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32]),
        "orc_ck_free": (None, [C.c_void_p]),
        "orc_ck_insert": (C.c_uint64, [C.c_void_p, _u32p, _u32p, C.c_uint64, C.c_void_p]),
        "orc_ck_insert_mt": (C.c_uint64, [C.c_void_p, _u32p, _u32p, C.c_uint64, C.c_int]),
        "orc_ck_find": (None, [C.c_void_p, _u32p, _u32p, C.c_uint64, C.c_int]),
        "orc_ck_erase": (None, [C.c_void_p, _u32p, C.c_uint64]),
        "orc_ck_resize_up": (C.c_int, [C.c_void_p]),
        "orc_ck_resize_down": (C.c_int, [C.c_void_p]),
        "orc_ck_pick_up": (C.c_int, [C.c_void_p]),
        "orc_ck_pick_down": (C.c_int, [C.c_void_p]),
        "orc_ck_capacity": (C.c_uint64, [C.c_void_p]),
        "orc_ck_count": (C.c_uint64, [C.c_void_p]),
        "orc_ck_dropped": (C.c_uint64, [C.c_void_p]),
        "orc_ck_layout": (None, [C.c_void_p, _u32p]),
        "orc_ck_export": (C.c_uint64, [C.c_void_p, _u32p, _u32p]),
        "orc_ck_subtable": (C.c_void_p, [C.c_void_p, C.c_uint32]),
        "orc_map_new": (C.c_void_p, [C.c_uint64]),
        "orc_map_free": (None, [C.c_void_p]),
        "orc_map_size": (C.c_uint64, [C.c_void_p]),
        "orc_map_apply": (None, [C.c_void_p, _u8p, _u64p, _u64p, C.c_uint64, _u64p, _u8p]),
        "orc_map_export": (C.c_uint64, [C.c_void_p, _u64p, _u64p]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


# ---------------------------------------------------------------- generators
class MT19937:
    """MT19937 stream (GPU/dyhash/mt19937ar.cpp), seeded like the reference."""

    def __init__(self, seed: int = 10327):
        self.st = _MT()
        lib().orc_mt_seed(C.byref(self.st), seed & 0xFFFFFFFF)

    def u32(self) -> int:
        return lib().orc_mt_u32(C.byref(self.st))

    def u31(self) -> int:
        return lib().orc_mt_u31(C.byref(self.st))

    def real1(self) -> float:
        return lib().orc_mt_real1(C.byref(self.st))

    def fill_u32(self, n: int) -> np.ndarray:
        out = np.empty(n, np.uint32)
        lib().orc_mt_fill_u32(C.byref(self.st), out, n)
        return out

    def unique_ref(self, n: int, max_number: int = 0xFFFFFFFE) -> np.ndarray:
        """GenerateUniqueRandomNumbers (random_numbers.cpp:26-77): 31-bit draws."""
        out = np.empty(n, np.uint32)
        if not lib().orc_gen_unique_ref(C.byref(self.st), out, n, max_number):
            raise MemoryError("orc_gen_unique_ref")
        return out

    def unique_full(self, n: int) -> np.ndarray:
        """Unique keys uniform in [1, 2^32-2] (same procedure, 32-bit draws)."""
        out = np.empty(n, np.uint32)
        if not lib().orc_gen_unique_full(C.byref(self.st), out, n):
            raise MemoryError("orc_gen_unique_full")
        return out

    def shuffle(self, a: np.ndarray) -> None:
        assert a.dtype == np.uint32 and a.flags.c_contiguous
        lib().orc_shuffle(C.byref(self.st), a.size, a)

    def queries(self, size: int, failure_rate: float, pool: np.ndarray) -> np.ndarray:
        """GenerateQueries (random_numbers.cpp:96-117); pool holds 2*size keys."""
        assert pool.dtype == np.uint32 and pool.size >= 2 * size
        q = np.empty(size, np.uint32)
        lib().orc_gen_queries(C.byref(self.st), size, failure_rate, pool, q)
        return q


# ------------------------------------------------------------------- hashing
def hash_fn(i: int, k: int) -> int:
    return getattr(lib(), "orc_hash%d" % i)(k)


def fold64(k: int) -> int:
    return lib().orc_fold64(k)


def bucket_of(hkey: int, t: int, nbuckets: int) -> int:
    return lib().orc_bucket_of(hkey, t, nbuckets)


def pair_of(hkey: int, d: int = 4):
    p = lib().orc_choose_hash(hkey, d)
    return p, lib().orc_pos1(p, d), lib().orc_pos2(p, d)


def hash_batch(keys: np.ndarray, d: int, nbuckets):
    keys = np.ascontiguousarray(keys, np.uint32)
    nb = np.ascontiguousarray(np.asarray(nbuckets, np.uint32))
    n = keys.size
    t1, b1, t2, b2 = (np.empty(n, np.uint32) for _ in range(4))
    lib().orc_hash_batch(keys, n, d, nb, t1, b1, t2, b2)
    return t1, b1, t2, b2


def next_prime(n: int) -> int:
    return lib().orc_next_prime(n)


def subtable_buckets(size: int, d: int = 4, slots: int = 16) -> int:
    return lib().orc_subtable_buckets(size, d, slots)


# ------------------------------------------------------ reference cuckoo table
class RefCuckoo:
    """The reference's table (GPU/dyhash/api.cpp + cuckoo.cu) on the CPU."""

    def __init__(self, size: int, d: int = 4, slots: int = 16, max_evict: int = 15):
        self.d, self.slots = d, slots
        self.h = lib().orc_ck_new(size, d, slots, max_evict)
        if not self.h:
            raise MemoryError("orc_ck_new")

    def close(self):
        if self.h:
            lib().orc_ck_free(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def insert(self, k, v, counts: bool = False, threads: int = 1):
        k = np.ascontiguousarray(k, np.uint32)
        v = np.ascontiguousarray(v, np.uint32)
        if threads > 1:
            return lib().orc_ck_insert_mt(self.h, k, v, k.size, threads)
        if counts:
            c = np.zeros(k.size, np.int32)
            f = lib().orc_ck_insert(self.h, k, v, k.size, c.ctypes.data)
            return f, c
        return lib().orc_ck_insert(self.h, k, v, k.size, None)

    def find(self, k, threads: int = 1) -> np.ndarray:
        k = np.ascontiguousarray(k, np.uint32)
        out = np.empty(k.size, np.uint32)
        lib().orc_ck_find(self.h, k, out, k.size, threads)
        return out

    def erase(self, k) -> None:
        k = np.ascontiguousarray(k, np.uint32)
        lib().orc_ck_erase(self.h, k, k.size)

    def resize_up(self) -> int:
        return lib().orc_ck_resize_up(self.h)

    def resize_down(self) -> int:
        return lib().orc_ck_resize_down(self.h)

    def pick_up(self) -> int:
        return lib().orc_ck_pick_up(self.h)

    def pick_down(self) -> int:
        return lib().orc_ck_pick_down(self.h)

    @property
    def capacity(self) -> int:
        return lib().orc_ck_capacity(self.h)

    @property
    def dropped(self) -> int:
        return lib().orc_ck_dropped(self.h)

    def count(self) -> int:
        return lib().orc_ck_count(self.h)

    def layout(self) -> np.ndarray:
        nb = np.zeros(self.d, np.uint32)
        lib().orc_ck_layout(self.h, nb)
        return nb

    def subtable(self, i: int) -> np.ndarray:
        nb = int(self.layout()[i])
        p = lib().orc_ck_subtable(self.h, i)
        buf = (C.c_uint64 * (nb * self.slots)).from_address(p)
        return np.ctypeslib.as_array(buf).copy().reshape(nb, self.slots)

    def export(self):
        n = self.count()
        k = np.empty(max(n, 1), np.uint32)
        v = np.empty(max(n, 1), np.uint32)
        c = lib().orc_ck_export(self.h, k, v)
        return k[:c], v[:c]


# -------------------------------------------------------------- semantic map
class Map:
    """Key->value semantics: upsert, batch-order duplicate rule, erase counts."""

    def __init__(self, hint: int = 1024):
        self.h = lib().orc_map_new(hint)
        if not self.h:
            raise MemoryError("orc_map_new")

    def close(self):
        if self.h:
            lib().orc_map_free(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __len__(self):
        return lib().orc_map_size(self.h)

    def apply(self, ops, keys, vals=None):
        keys = np.ascontiguousarray(keys, np.uint64)
        n = keys.size
        ops = np.ascontiguousarray(np.broadcast_to(np.asarray(ops, np.uint8), (n,)))
        vals = np.zeros(n, np.uint64) if vals is None else np.ascontiguousarray(vals, np.uint64)
        out_v = np.empty(n, np.uint64)
        out_h = np.empty(n, np.uint8)
        lib().orc_map_apply(self.h, ops, keys, vals, n, out_v, out_h)
        return out_v, out_h.astype(bool)

    def insert(self, keys, vals):
        return self.apply(OP_INSERT, keys, vals)

    def find(self, keys):
        return self.apply(OP_FIND, keys)

    def erase(self, keys):
        return self.apply(OP_ERASE, keys)

    def export(self):
        n = len(self)
        k = np.empty(max(n, 1), np.uint64)
        v = np.empty(max(n, 1), np.uint64)
        c = lib().orc_map_export(self.h, k, v)
        order = np.argsort(k[:c], kind="stable")
        return k[:c][order], v[:c][order]
