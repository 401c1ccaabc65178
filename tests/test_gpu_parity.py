"""GPU parity: the CUDA table through the C ABI against the oracle.

Every check is exact: find values and hit bits, erase counts and erased
bits, and the table's full key->value contents after every batch equal the
oracle's map semantics (upsert; last occurrence wins within an insert batch;
first occurrence removes within an erase batch; key 0 is never stored).
The placement test also checks that every resident key sits in a bucket the
reference's hash functions give it (GPU/dyhash/cuckoo.cu:76-90, :190-213).
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import (assert_same_contents, find_and_compare, first_probe_table, to_dev,
                           to_host, unique_u32, unique_u64)

pytestmark = pytest.mark.gpu


def _dg():
    import databases_gpu_gb300 as dg
    return dg


def _bits_np(bits, n):
    return _dg().unpack_bits(bits, n)


# ------------------------------------- the reference test scale (2^20 keys)
def test_config1_insert_find_erase_refind():
    """2^20 unique u32 keys at load factor 0.85, 2^20 finds (50% hits),
    2^19 erases, re-find; contents checked after every batch."""
    n = 1 << 20
    pool = unique_u32(2 * n, seed=10327)
    keys, miss = pool[:n], pool[n:]
    vals = (np.arange(n, dtype=np.uint32) * 3 + 4) & 0x7FFFFFFF
    t = _dg().DyCuckoo(int(n / 0.85), auto_resize=False)
    m = O.Map(n)
    st = t.insert(to_dev(keys), to_dev(vals))
    m.insert(keys, vals)
    assert st["inserted"] == n and st["updated"] == 0
    assert_same_contents(t, m, "after insert")
    mt = O.MT19937(4242)
    q = mt.queries(n, 0.5, np.concatenate([keys, miss]).copy())
    hits = find_and_compare(t, m, q, "find 50%")
    assert hits.sum() == n // 2
    er = keys[: n // 2].copy()
    mt.shuffle(er)
    bits = __import__("torch").zeros(n // 2 // 32, dtype=__import__("torch").int32, device="cuda")
    cnt = t.erase(to_dev(er), erased_bits=bits)
    _, oh = m.erase(er)
    assert cnt == n // 2 == int(oh.sum())
    assert np.array_equal(_bits_np(bits, n // 2), oh)
    assert_same_contents(t, m, "after erase")
    find_and_compare(t, m, q, "re-find")
    t.close()


# ------------------------------------------------------ batch-order rules
def test_repeated_keys_last_insert_wins():
    rng = np.random.default_rng(1)
    n = 200_000
    keys = rng.integers(1, 5000, n, dtype=np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    t = _dg().DyCuckoo(20000)
    m = O.Map()
    st = t.insert(to_dev(keys), to_dev(vals))
    m.insert(keys, vals)
    assert st["superseded"] == n - np.unique(keys).size
    assert_same_contents(t, m, "dup insert")
    # second batch: upserts of present keys plus new ones
    k2 = rng.integers(1, 10000, n, dtype=np.uint32)
    v2 = np.arange(n, dtype=np.uint32) + 7
    st = t.insert(to_dev(k2), to_dev(v2))
    m.insert(k2, v2)
    assert st["updated"] > 0 and st["inserted"] > 0
    assert_same_contents(t, m, "upsert batch")
    t.close()


def test_repeated_keys_first_erase_removes():
    import torch
    rng = np.random.default_rng(2)
    keys = unique_u32(50_000, seed=7)
    t = _dg().DyCuckoo(100_000)
    m = O.Map()
    t.insert(to_dev(keys), to_dev(keys))
    m.insert(keys, keys)
    er = np.concatenate([rng.choice(keys, 30_000), rng.integers(1, 1 << 32, 2000, dtype=np.uint64).astype(np.uint32)])
    rng.shuffle(er)
    bits = torch.zeros((er.size + 31) // 32, dtype=torch.int32, device="cuda")
    cnt = t.erase(to_dev(er), erased_bits=bits, no_resize=True)
    _, oh = m.erase(er)
    assert cnt == int(oh.sum())
    assert np.array_equal(_bits_np(bits, er.size), oh)
    assert_same_contents(t, m, "dup erase")
    t.close()


@pytest.mark.parametrize("key_bytes", [4, 8])
def test_repeats_in_large_chunks_use_the_winner_bits(key_bytes):
    """Insert and erase chunks of 2^21 + 5 ops, whose dedup tables (2^22
    cells) get the winners pass, against chunks of 2^16 ops, which look
    their winners up in the dedup table: keys repeat within the batch (a
    pool of 2^20 keys), the last insert of a key wins and the first erase
    removes it; counts, erase bits and contents equal the oracle's."""
    import torch
    rng = np.random.default_rng(91 + key_bytes)
    npk = np.uint32 if key_bytes == 4 else np.uint64
    pool = (unique_u32(1 << 20, seed=92) if key_bytes == 4 else
            unique_u64(1 << 20, seed=92)).astype(npk)
    n = (1 << 21) + 5
    t = _dg().DyCuckoo(1 << 21, key_bytes=key_bytes, value_bytes=key_bytes)
    m = O.Map()
    keys = pool[rng.integers(0, pool.size, n)]
    vals = rng.integers(1, 1 << 30, n).astype(npk)
    st = t.insert(to_dev(keys), to_dev(vals))
    _, oh = m.insert(keys.astype(np.uint64), vals.astype(np.uint64))
    assert st["inserted"] == int((~oh).sum()) and st["superseded"] > 0
    assert_same_contents(t, m, "large insert with repeats")
    for size in (n, 1 << 16):
        ek = pool[rng.integers(0, pool.size, size)]
        ek[::97] = rng.integers(1, 1 << 30, ek[::97].size).astype(npk)  # misses, mostly
        bits = torch.zeros((size + 31) // 32, dtype=torch.int32, device="cuda")
        cnt = t.erase(to_dev(ek), erased_bits=bits, no_resize=True)
        _, eh = m.erase(ek.astype(np.uint64))
        assert cnt == int(eh.sum())
        assert np.array_equal(_bits_np(bits, size), eh), "erase of %d: bits differ" % size
        assert_same_contents(t, m, "erase of %d with repeats" % size)
        re = pool[rng.integers(0, pool.size, size)]
        rv = rng.integers(1, 1 << 30, size).astype(npk)
        t.insert(to_dev(re), to_dev(rv))
        m.insert(re.astype(np.uint64), rv.astype(np.uint64))
        assert_same_contents(t, m, "re-insert of %d with repeats" % size)
    t.close()


def test_key_zero_is_never_stored():
    keys = np.array([0, 5, 0, 9, 11], np.uint32)
    vals = np.array([1, 2, 3, 4, 5], np.uint32)
    t = _dg().DyCuckoo(1000)
    m = O.Map()
    st = t.insert(to_dev(keys), to_dev(vals))
    m.insert(keys, vals)
    assert st["rejected"] == 2 and st["inserted"] == 3
    assert_same_contents(t, m)
    find_and_compare(t, m, np.array([0, 5, 9, 11, 12], np.uint32))
    assert t.erase(to_dev(np.array([0, 0], np.uint32))) == 0
    t.close()


def test_empty_and_ragged_batches():
    t = _dg().DyCuckoo(1000)
    m = O.Map()
    import torch
    e = torch.empty(0, dtype=torch.int32, device="cuda")
    t.insert(e, e)
    out, _ = t.find(e)
    assert out.numel() == 0
    for n in (1, 31, 33, 1000, 4097):
        k = unique_u32(n, seed=n)
        t.insert(to_dev(k), to_dev(k + 1))
        m.insert(k, k + 1)
        find_and_compare(t, m, k, "ragged %d" % n)
    assert_same_contents(t, m)
    t.close()


# ---------------------------------------------------------------- structure
@pytest.mark.parametrize("bucket_bytes", [32, 64, 128])
@pytest.mark.parametrize("d", [2, 3, 4, 5, 6])
def test_placement_follows_reference_hashes(bucket_bytes, d):
    n = 60_000
    keys = unique_u32(n, seed=d * 131 + bucket_bytes)
    t = _dg().DyCuckoo(int(n / 0.8), num_subtables=d, bucket_bytes=bucket_bytes, auto_resize=False)
    m = O.Map()
    t.insert(to_dev(keys), to_dev(keys ^ np.uint32(0x5A5A5A5A)))
    m.insert(keys, keys ^ np.uint32(0x5A5A5A5A))
    assert_same_contents(t, m, "d=%d sb=%d" % (d, bucket_bytes))
    nb = t.layout()
    seen = 0
    for s in range(d):
        sub = t.subtable(s)  # (buckets, slots) of key | value << 32
        kk = (sub & np.uint64(0xFFFFFFFF)).astype(np.uint32)
        b_idx, _ = np.nonzero(kk)
        rk = kk[kk != 0]
        seen += rk.size
        t1, b1, t2, b2 = O.hash_batch(rk, d, nb)
        in1 = (t1 == s) & (b1 == b_idx)
        in2 = (t2 == s) & (b2 == b_idx)
        assert np.all(in1 | in2), "subtable %d holds keys outside their buckets" % s
    assert seen == n
    find_and_compare(t, m, keys[:5000])
    t.close()


@pytest.mark.parametrize("bucket_bytes,floor", [(32, 0.75), (128, 0.9)])
def test_first_probe_serves_most_hits(bucket_bytes, floor):
    """Finds probe the first-probe bucket first; the insert policy keeps most
    keys there (so a hit costs one bucket read)."""
    n = 1 << 18
    keys = unique_u32(n, seed=99)
    t = _dg().DyCuckoo(int(n / 0.9), bucket_bytes=bucket_bytes, auto_resize=False)
    t.insert(to_dev(keys), to_dev(keys))
    nb = t.layout()
    first = 0
    for s in range(4):
        sub = t.subtable(s)
        kk = (sub & np.uint64(0xFFFFFFFF)).astype(np.uint32)
        rk = kk[kk != 0]
        first += int((first_probe_table(rk, 4, nb) == s).sum())
    frac = first / n
    assert frac > floor, frac
    t.close()


def _fp_bit(keys: np.ndarray) -> np.ndarray:
    """Displacement fingerprint bit of 4-byte keys: 1 << ((k * 0x9E3779B1 mod
    2^32) >> 26)."""
    with np.errstate(over="ignore"):
        f = (keys.astype(np.uint32) * np.uint32(0x9E3779B1)) >> np.uint32(26)
    return np.uint64(1) << f.astype(np.uint64)


def _check_overflow_bits(t, d=4):
    """Every key stored in its second bucket has its fingerprint bit set in
    the metadata word of its first-probe bucket (128-byte buckets)."""
    nb = t.layout()
    metas = [t.subtable(s, with_meta=True)[:, -1] for s in range(d)]
    bad = 0
    for s in range(d):
        sub = t.subtable(s)
        kk = (sub & np.uint64(0xFFFFFFFF)).astype(np.uint32)
        b_idx, _ = np.nonzero(kk)
        rk = kk[kk != 0]
        t1, b1, t2, b2 = O.hash_batch(rk, d, nb)
        first_t = first_probe_table(rk, d, nb)
        first_b = np.where(first_t == t1, b1, b2)
        second = first_t != s
        for ft in range(d):
            sel = second & (first_t == ft)
            if sel.any():
                bits = metas[ft][first_b[sel]] & _fp_bit(rk[sel])
                bad += int((bits == 0).sum())
    return bad


def test_overflow_bits_cover_every_displaced_key():
    n = 1 << 18
    keys = unique_u32(2 * n, seed=4321)
    t = _dg().DyCuckoo(int(n / 0.9), auto_resize=False)
    m = O.Map()
    t.insert(to_dev(keys[:n]), to_dev(keys[:n]))
    m.insert(keys[:n], keys[:n])
    assert _check_overflow_bits(t) == 0
    t.erase(to_dev(keys[: n // 3]), no_resize=True)
    m.erase(keys[: n // 3])
    t.insert(to_dev(keys[n: n + n // 3]), to_dev(keys[n: n + n // 3]))
    m.insert(keys[n: n + n // 3], keys[n: n + n // 3])
    assert _check_overflow_bits(t) == 0
    t.resize_up()
    assert _check_overflow_bits(t) == 0
    t.resize_down()
    t.resize_down()
    assert _check_overflow_bits(t) == 0
    assert_same_contents(t, m, "after bit checks")
    find_and_compare(t, m, keys, "misses skip the second probe only when safe")
    t.close()


# ---------------------------------------------------------------- resizing
@pytest.mark.parametrize("bucket_bytes,slots", [(32, 4), (128, 15)])
def test_resize_sequence_matches_reference_policy(bucket_bytes, slots):
    """Initial bucket counts follow the reference sizing rule (api.cpp:46-56)
    with this table's entry slots per bucket; each resize doubles or halves
    the subtable the reference's choice rules name (api.cpp:115-122, :147-153,
    pinned against the reference in test_oracle_golden)."""
    n = 100_000
    keys = unique_u32(n, seed=5)
    vals = np.arange(n, dtype=np.uint32)
    t = _dg().DyCuckoo(n * 2, bucket_bytes=bucket_bytes, auto_resize=False)
    nb = np.array([O.subtable_buckets(n * 2, 4, slots)] * 4, np.uint32)
    assert t.layout() == [int(x) for x in nb]
    L = O.lib()
    m = O.Map()
    t.insert(to_dev(keys), to_dev(vals))
    m.insert(keys, vals)
    for step in range(5):
        t.resize_up()
        i = L.orc_pick_up_nb(nb, 4)
        nb[i] *= 2
        assert t.layout() == [int(x) for x in nb], "up %d" % step
        assert_same_contents(t, m, "after up %d" % step)
        find_and_compare(t, m, keys[::7], "find after up %d" % step)
    for step in range(7):
        t.resize_down()
        i = L.orc_pick_down_nb(nb, 4)
        nb[i] = nb[i] // 2 if nb[i] % 2 == 0 else (nb[i] + 1) // 2
        assert t.layout() == [int(x) for x in nb], "down %d" % step
        assert_same_contents(t, m, "after down %d" % step)
        find_and_compare(t, m, keys[::7], "find after down %d" % step)
    t.close()


def test_downsize_into_full_subtables_never_drops():
    """Halve subtables of a dense table: merged buckets overflow and the
    leftovers are walked into other subtables (the reference drops them,
    cuckoo.cu:714-722); an upsize happens when even that fails."""
    n = 150_000
    keys = unique_u32(n, seed=77)
    t = _dg().DyCuckoo(int(n / 0.75), auto_resize=False)
    m = O.Map()
    t.insert(to_dev(keys), to_dev(keys + 3))
    m.insert(keys, keys + 3)
    for _ in range(3):
        t.resize_down()
        assert_same_contents(t, m, "dense downsize")
    find_and_compare(t, m, keys, "after dense downsizes")
    t.close()


def test_pool_reserve_then_resizes_keep_everything():
    """dyc_pool_reserve maps memory into the allocation pool; the resizes that
    follow take their buffers from it and keep every key."""
    n = 200_000
    keys = unique_u32(n, seed=31)
    t = _dg().DyCuckoo(n, auto_resize=False)
    _dg().pool_reserve(256 << 20)
    m = O.Map()
    t.insert(to_dev(keys), to_dev(keys ^ np.uint32(0x5A5A)))
    m.insert(keys, keys ^ np.uint32(0x5A5A))
    for _ in range(3):
        t.resize_up()
    t.resize_down()
    assert_same_contents(t, m, "resizes after a pool reserve")
    find_and_compare(t, m, keys, "after resizes")
    t.close()


def test_eviction_overflow_upsizes_and_keeps_everything():
    n = 50_000
    keys = unique_u32(n, seed=8)
    t = _dg().DyCuckoo(64, max_evictions=1, auto_resize=False)
    m = O.Map()
    cap0 = t.capacity
    st = t.insert(to_dev(keys), to_dev(keys * np.uint32(3)))
    m.insert(keys, keys * np.uint32(3))
    assert st["overflowed"] > 0 and st["resizes_up"] > 0
    assert t.capacity > cap0
    assert_same_contents(t, m, "overflow")
    t.close()


def test_auto_resize_thresholds():
    n = 1 << 16
    keys = unique_u32(4 * n, seed=12)
    t = _dg().DyCuckoo(n, auto_resize=True, min_downsize_capacity=0)
    m = O.Map()
    for i in range(4):
        k = keys[i * n:(i + 1) * n]
        t.insert(to_dev(k), to_dev(k))
        m.insert(k, k)
        assert t.size <= 0.8 * t.capacity + 1
    assert_same_contents(t, m, "grown")
    for i in range(4):
        k = keys[i * n:(i + 1) * n]
        t.erase(to_dev(k))
        m.erase(k)
        assert_same_contents(t, m, "shrinking %d" % i)
    assert t.size == 0
    t.close()


# ---------------------------------------------------------------- 8-byte keys
@pytest.mark.parametrize("value_bytes", [8, 4])
@pytest.mark.parametrize("bucket_bytes", [32, 64, 128])
def test_u64_keys(value_bytes, bucket_bytes):
    import torch
    n = 100_000
    keys = unique_u64(n, seed=bucket_bytes + value_bytes)
    vmask = np.uint64(0xFFFFFFFF) if value_bytes == 4 else np.uint64(0xFFFFFFFFFFFFFFFF)
    vals = (keys * np.uint64(3)) & vmask
    vals_dev = vals.astype(np.uint32) if value_bytes == 4 else vals
    t = _dg().DyCuckoo(int(n / 0.8), key_bytes=8, value_bytes=value_bytes,
                       bucket_bytes=bucket_bytes, auto_resize=False)
    m = O.Map()
    t.insert(to_dev(keys), to_dev(vals_dev))
    m.insert(keys, vals)
    assert_same_contents(t, m, "u64 insert")
    q = np.concatenate([keys[: n // 2], unique_u64(n // 2, seed=991)])
    find_and_compare(t, m, q, "u64 find")
    er = keys[::3]
    bits = torch.zeros((er.size + 31) // 32, dtype=torch.int32, device="cuda")
    cnt = t.erase(to_dev(er), erased_bits=bits)
    _, oh = m.erase(er)
    assert cnt == int(oh.sum())
    assert_same_contents(t, m, "u64 erase")
    t.resize_up()
    t.resize_down()
    t.resize_down()
    assert_same_contents(t, m, "u64 resizes")
    # keys that share their low or high halves (fold collisions)
    k2 = np.array([(1 << 32) | 5, (2 << 32) | 5, 5, (5 << 32), (7 << 32) | 7], np.uint64)
    v2 = np.arange(5, dtype=np.uint64) + 1
    t.insert(to_dev(k2), to_dev(v2.astype(np.uint32) if value_bytes == 4 else v2))
    m.insert(k2, v2)
    assert_same_contents(t, m, "u64 fold collisions")
    t.close()


# ------------------------------------------------ host-buffer C ABI forms
def test_host_forms_match_device_forms():
    n = 300_000
    keys = unique_u32(2 * n, seed=21)
    t = _dg().DyCuckoo(n * 2)
    m = O.Map()
    t.insert_host(keys[:n], keys[:n] + 1)
    m.insert(keys[:n], keys[:n] + 1)
    out = np.zeros(2 * n, np.uint32)
    bits = np.zeros((2 * n + 31) // 32, np.uint32)
    t.find_host(keys, out, bits)
    ov, oh = m.find(keys)
    assert np.array_equal(out.astype(np.uint64), ov)
    assert np.array_equal(_bits_np(bits, 2 * n), oh)
    cnt = t.erase_host(keys[n // 2: n + n // 2])
    _, eh = m.erase(keys[n // 2: n + n // 2])
    assert cnt == int(eh.sum())
    assert_same_contents(t, m, "host forms")
    t.close()


@pytest.mark.parametrize("chunks", [3, 5])
def test_host_find_pipeline_chunk_schedule(chunks):
    """A host find spanning several pipeline chunks on all three streams
    (each stream reused when there are five) and a ragged last chunk: values
    and hit bits equal a device find of the same keys."""
    import torch
    n = chunks * (1 << 22) + 4133
    keys = unique_u32(n, seed=29)
    t = _dg().DyCuckoo(n)
    half = n // 2
    t.insert(to_dev(keys[:half]), to_dev(keys[:half] ^ np.uint32(0x1234)))
    out = np.zeros(n, np.uint32)
    bits = np.zeros((n + 31) // 32, np.uint32)
    t.find_host(keys, out, bits)
    dv, db = t.find(to_dev(keys))
    assert np.array_equal(out, to_host(dv, 4))
    assert np.array_equal(bits.view(np.int32), db.cpu().numpy())
    assert int(_bits_np(bits, n).sum()) == half
    t.close()


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_l2_residency_modes_give_the_same_results(mode):
    """dyc_config.l2_resident only changes the L2 cache policy of the bucket
    reads (evict_last hints in mode 2, plain loads otherwise) and of find's
    streaming keys and results: inserts, finds (hits and misses), erases and
    the contents match the oracle in every mode."""
    import databases_gpu_gb300 as dg
    n = 1 << 16
    pool = unique_u32(2 * n, seed=91)
    keys, vals = pool[:n], np.arange(3, n + 3, dtype=np.uint32)
    t = dg.DyCuckoo(int(n / 0.85), l2_resident=mode)
    m = O.Map(n)
    t.insert(to_dev(keys), to_dev(vals))
    m.insert(keys, vals)
    find_and_compare(t, m, pool, "find, l2_resident=%d" % mode)
    assert t.erase(to_dev(keys[: n // 3])) == n // 3
    m.erase(keys[: n // 3])
    find_and_compare(t, m, pool, "find after erase, l2_resident=%d" % mode)
    assert_same_contents(t, m, "contents, l2_resident=%d" % mode)
    t.close()


@pytest.mark.parametrize("key_bytes", [4, 8])
def test_many_chunks_with_repeats_match_oracle(key_bytes):
    """Inserts and erases split into many chunks (tables made with a
    4096-op chunk, dyc_debug_inject): keys repeat within chunks and across
    them, the table grows between chunks (auto resize), and erases include
    misses. Every erase bit, the counts, the finds and the contents equal
    the oracle's."""
    import databases_gpu_gb300 as dg
    from databases_gpu_gb300 import _lib
    from tests.helpers import unique_u64
    L = _lib.lib()
    assert L.dyc_debug_inject(_lib.INJECT_CHUNK_OPS, 4096) == 0
    try:
        t = dg.DyCuckoo(1 << 12, key_bytes=key_bytes, value_bytes=key_bytes)
    finally:
        L.dyc_debug_inject(_lib.INJECT_RESET, 0)
    rng = np.random.default_rng(61)
    pool = (unique_u32(60000, seed=62) if key_bytes == 4 else unique_u64(60000, seed=62))
    npk = np.uint32 if key_bytes == 4 else np.uint64
    m = O.Map()
    for r in range(3):
        keys = pool[rng.integers(0, 40000 + 10000 * r, 50000)].astype(npk)
        vals = rng.integers(1, 1 << 30, keys.size).astype(npk)
        st = t.insert(to_dev(keys), to_dev(vals))
        _, oh = m.insert(keys.astype(np.uint64), vals.astype(np.uint64))
        assert st["inserted"] == int((~oh).sum()), (r, st)
        assert t.size == len(m), (r, t.size, len(m))
        ek = pool[rng.integers(0, 60000, 30000)].astype(npk)  # repeats and misses
        import torch
        bits = torch.zeros((ek.size + 31) // 32, dtype=torch.int32, device="cuda")
        cnt = t.erase(to_dev(ek), erased_bits=bits)
        _, eh = m.erase(ek.astype(np.uint64))
        assert cnt == int(eh.sum()), (r, cnt, int(eh.sum()))
        gh = dg.unpack_bits(bits, ek.size)
        assert np.array_equal(gh, eh), "round %d: %d erase bits differ" % (r, int((gh != eh).sum()))
        find_and_compare(t, m, pool, "chunks round %d" % r)
    assert_same_contents(t, m, "chunked inserts and erases")
    t.close()
