"""Generate tests/golden/reference_kat.npz from the reference's own code.

Runs in the build container, where the reference tree exists: it builds
oracle/_ref/libref_host.so (oracle/build_ref.py compiles the reference's
hash functions, pair maps, makeEntry, sizing, resize target choice, MT19937
and key generators from their sources) and records their outputs on fixed
inputs. The committed fixture is what the CPU tests pin the oracle against;
nothing at test time reads the reference tree.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build_ref  # noqa: E402

OUT = os.path.join(HERE, "reference_kat.npz")


def main() -> None:
    path = build_ref.build()
    if path is None:
        raise SystemExit("reference tree not present; cannot regenerate golden vectors")
    L = C.CDLL(path)
    u32 = C.c_uint32
    for name in ["ref_hash1", "ref_hash2", "ref_hash3", "ref_hash4", "ref_hash5",
                 "ref_choose_hash4", "ref_pos1_4", "ref_pos2_4", "ref_next_prime",
                 "ref_subtable_buckets"]:
        getattr(L, name).restype = u32
        getattr(L, name).argtypes = [u32]
    L.ref_hash_function.restype = u32
    L.ref_hash_function.argtypes = [u32, u32, u32]
    L.ref_get_pos4.restype = u32
    L.ref_get_pos4.argtypes = [u32, u32]
    for name in ["ref_choose_hash_d", "ref_pos1_d", "ref_pos2_d"]:
        getattr(L, name).restype = u32
        getattr(L, name).argtypes = [u32, u32]
    L.ref_make_entry.restype = C.c_uint64
    L.ref_make_entry.argtypes = [u32, u32]
    L.ref_is_prime.restype = C.c_int
    L.ref_is_prime.argtypes = [C.c_int]
    L.ref_pick_up.restype = u32
    L.ref_pick_up.argtypes = [C.POINTER(u32)]
    L.ref_pick_down.restype = u32
    L.ref_pick_down.argtypes = [C.POINTER(u32)]
    init = L._Z12init_genrandm
    init.argtypes = [C.c_ulong]
    g32 = L._Z13genrand_int32v
    g32.restype = C.c_ulong
    gen_unique = L._Z27GenerateUniqueRandomNumbersPjjj
    gen_unique.restype = C.c_bool
    gen_unique.argtypes = [C.POINTER(u32), u32, u32]
    gen_q = L._Z15GenerateQueriesjfPjS_
    gen_q.argtypes = [u32, C.c_float, C.POINTER(u32), C.POINTER(u32)]

    out = {}
    # ---- MT19937 stream as the reference tests seed it (Main_backup_0910.cpp:180)
    init(10327)
    out["mt_10327"] = np.array([g32() for _ in range(2000)], np.uint32)
    init(5489)
    out["mt_5489"] = np.array([g32() for _ in range(1000)], np.uint32)

    # ---- hash inputs: edge values plus an MT-drawn spread
    init(99991)
    keys = np.array([0, 1, 2, 3, 11, 255, 256, 65535, 65536, 0x7FFFFFFF, 0x80000000,
                     0xFFFFFFFE, 0xFFFFFFFF, 294967291, 294967290, 4294967291]
                    + [g32() for _ in range(1008)], np.uint32)
    out["hash_keys"] = keys
    for i in range(1, 6):
        f = getattr(L, "ref_hash%d" % i)
        out["hash%d" % i] = np.array([f(int(k)) for k in keys], np.uint32)
    nbs = np.array([1, 2, 38, 19290, 262144, 4660394, 18641578], np.uint32)
    out["hf_nbuckets"] = nbs
    hf = np.zeros((4, nbs.size, keys.size), np.uint32)
    for t in range(4):
        for j, nb in enumerate(nbs):
            hf[t, j] = [L.ref_hash_function(int(k), t, int(nb)) for k in keys]
    out["hash_function"] = hf
    out["choose4"] = np.array([L.ref_choose_hash4(int(k)) for k in keys], np.uint32)
    out["pos1_4"] = np.array([L.ref_pos1_4(p) for p in range(6)], np.uint32)
    out["pos2_4"] = np.array([L.ref_pos2_4(p) for p in range(6)], np.uint32)
    out["get_pos4"] = np.array([[L.ref_get_pos4(p, pre) for pre in (0, 1, 2, 3, 100)]
                                for p in range(6)], np.uint32)
    for d, npairs in ((2, 2), (3, 3), (5, 10)):
        out["choose_d%d" % d] = np.array([L.ref_choose_hash_d(d, int(k)) for k in keys],
                                         np.uint32)
        out["pos1_d%d" % d] = np.array([L.ref_pos1_d(d, p) for p in range(npairs)], np.uint32)
        out["pos2_d%d" % d] = np.array([L.ref_pos2_d(d, p) for p in range(npairs)], np.uint32)

    # ---- makeEntry with the `int` conversions of cuckoo_insert
    ek = np.array([1, 7, 12345, 0x7FFFFFFF, 0x80000000, 0xFFFFFFFE], np.uint32)
    ev = np.array([0, 1, 4, 0x7FFFFFFF, 0x80000000, 0xFFFFFFFF], np.uint32)
    out["entry_k"] = np.repeat(ek, ev.size)
    out["entry_v"] = np.tile(ev, ek.size)
    out["entry"] = np.array([L.ref_make_entry(int(a), int(b))
                             for a, b in zip(out["entry_k"], out["entry_v"])], np.uint64)

    # ---- sizing
    pr = np.arange(0, 5000, dtype=np.int64)
    out["is_prime"] = np.array([L.ref_is_prime(int(x)) for x in pr], np.int32)
    np_in = np.array([0, 1, 2, 3, 4, 100, 1000, 19275, 1 << 16, 4660337, 1 << 22],
                     np.uint32)
    out["next_prime_in"] = np_in
    out["next_prime"] = np.array([L.ref_next_prime(int(x)) for x in np_in], np.uint32)
    sizes = np.array([100, 110, 200, 1024, 1126, 4096, 1 << 16, 72089, 1 << 20, 1233618,
                      1 << 22, 2000000, 298261617, 4294967295], np.uint64)
    out["size_in"] = sizes
    out["subtable_buckets"] = np.array([L.ref_subtable_buckets(int(s)) for s in sizes],
                                       np.uint32)

    # ---- resize target choice
    layouts = np.array([[8, 8, 8, 8], [16, 8, 8, 8], [16, 16, 8, 8], [16, 16, 16, 8],
                        [8, 8, 8, 4], [8, 8, 4, 4], [8, 4, 4, 4], [16, 8, 8, 4]], np.uint32)
    out["layouts"] = layouts
    arr = (u32 * 4)
    out["pick_up"] = np.array([L.ref_pick_up(arr(*map(int, l))) for l in layouts], np.uint32)
    out["pick_down"] = np.array([L.ref_pick_down(arr(*map(int, l))) for l in layouts],
                                np.uint32)

    # ---- key generators: GenerateUniqueRandomNumbers and GenerateQueries
    for n in (100, 1024, 20000):
        init(10327)
        buf = (u32 * (2 * n))()
        assert gen_unique(buf, 2 * n, 0xFFFFFFFE)
        out["unique_10327_%d" % n] = np.frombuffer(buf, np.uint32).copy()
    init(4242)
    n = 5000
    pool = (u32 * (2 * n))()
    gen_unique(pool, 2 * n, 0xFFFFFFFE)
    out["queries_pool_before"] = np.frombuffer(pool, np.uint32).copy()
    q = (u32 * n)()
    gen_q(n, C.c_float(0.5), pool, q)
    out["queries_05"] = np.frombuffer(q, np.uint32).copy()
    out["queries_pool_after"] = np.frombuffer(pool, np.uint32).copy()

    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
