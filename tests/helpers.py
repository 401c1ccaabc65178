"""Shared helpers for the parity tests: seeded workloads, device transfer and
comparison against the oracle."""
from __future__ import annotations

import numpy as np

from oracle import oracle as O


def to_dev(a: np.ndarray):
    import torch
    a = np.ascontiguousarray(a)
    if a.dtype == np.uint32:
        a = a.view(np.int32)
    elif a.dtype == np.uint64:
        a = a.view(np.int64)
    return torch.from_numpy(a).cuda()


def to_host(t, unsigned_bytes: int) -> np.ndarray:
    a = t.cpu().numpy()
    return a.view(np.uint32 if unsigned_bytes == 4 else np.uint64)


def assert_same_contents(table, omap: O.Map, label: str = ""):
    k, v = table.export()
    kb = table.key_bytes
    gk = to_host(k, kb).astype(np.uint64)
    gv = to_host(v, table.value_bytes).astype(np.uint64)
    order = np.argsort(gk, kind="stable")
    gk, gv = gk[order], gv[order]
    ok_, ov_ = omap.export()
    assert gk.size == ok_.size, "%s: %d live entries on GPU, %d in oracle" % (label, gk.size, ok_.size)
    assert np.array_equal(gk, ok_), "%s: key sets differ" % label
    bad = np.nonzero(gv != ov_)[0]
    assert bad.size == 0, "%s: %d values differ, first key %d gpu %d oracle %d" % (
        label, bad.size, gk[bad[0]], gv[bad[0]], ov_[bad[0]])
    assert table.size == ok_.size, "%s: size counter %d vs %d" % (label, table.size, ok_.size)


def find_and_compare(table, omap: O.Map, queries: np.ndarray, label: str = ""):
    from databases_gpu_gb300 import unpack_bits
    out, bits = table.find(to_dev(queries))
    gv = to_host(out, table.value_bytes).astype(np.uint64)
    gh = unpack_bits(bits, queries.size)
    ov, oh = omap.find(queries.astype(np.uint64))
    assert np.array_equal(gh, oh), "%s: %d hit flags differ" % (label, int((gh != oh).sum()))
    bad = np.nonzero(gv != ov)[0]
    assert bad.size == 0, "%s: %d values differ" % (label, bad.size)
    return gh


def unique_u32(n: int, seed: int = 10327) -> np.ndarray:
    return O.MT19937(seed).unique_full(n)


def unique_u64(n: int, seed: int = 10327) -> np.ndarray:
    """n distinct nonzero 64-bit keys (splitmix64 of a seeded counter)."""
    with np.errstate(over="ignore"):  # wrapping 64-bit arithmetic is intended
        x = (np.arange(1, n + 1, dtype=np.uint64) + np.uint64(seed) * np.uint64(0x9E3779B97F4A7C15))
        x = x * np.uint64(0x9E3779B97F4A7C15)
        x ^= x >> np.uint64(30)
        x *= np.uint64(0xBF58476D1CE4E5B9)
        x ^= x >> np.uint64(27)
        x *= np.uint64(0x94D049BB133111EB)
        x ^= x >> np.uint64(31)
    x[x == 0] = np.uint64(1)
    return x  # splitmix64 finalizer is a bijection, so keys are distinct


def np_hash5(k: np.ndarray) -> np.ndarray:
    """get_hash5 of the reference (GPU/dyhash/cuckoo.cu:110-120), vectorised."""
    a = k.astype(np.uint32).copy()
    with np.errstate(over="ignore"):
        a -= a << np.uint32(6)
        a ^= a >> np.uint32(17)
        a -= a << np.uint32(9)
        a ^= a << np.uint32(4)
        a -= a << np.uint32(3)
        a ^= a << np.uint32(10)
        a ^= a >> np.uint32(15)
    return a


def first_probe_table(keys: np.ndarray, d: int, nbuckets) -> np.ndarray:
    """Subtable the CUDA table probes first for each key: the reference pair,
    ordered by bit 16 of hash5."""
    t1, _, t2, _ = O.hash_batch(keys, d, nbuckets)
    swap = (np_hash5(keys) >> np.uint32(16)) & np.uint32(1)
    return np.where(swap == 1, t2, t1)
