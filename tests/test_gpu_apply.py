"""GPU parity of mixed batches (dyc_apply) against the oracle's map, op by op.

For every op the value it saw (found / replaced / removed, 0 when absent) and
its hit bit (key present just before the op) must equal the oracle's, which
runs the same ops one at a time in index order; the table's full contents
must equal the oracle's after every batch. Cases: unique keys (resolved by
the op-order scatter pass), heavy repetition (segments replayed by one
thread), keys repeated tens to thousands of times (segments replayed by a
warp, or sorted by a block in shared-memory chunks merged in global memory),
key 0, u64 keys, batches that span several internal chunks, and
growth/shrink through the resize policy.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import assert_same_contents, to_dev, to_host, unique_u32, unique_u64

pytestmark = pytest.mark.gpu


def _dg():
    import databases_gpu_gb300 as dg
    return dg


def _apply_and_compare(t, m, ops, keys, vals, label, unique=False):
    out, bits = t.apply(to_dev(ops), to_dev(keys), to_dev(vals), unique=unique)
    gv = to_host(out, t.value_bytes).astype(np.uint64)
    gh = _dg().unpack_bits(bits, keys.size)
    ov, oh = m.apply(ops, keys.astype(np.uint64), vals.astype(np.uint64))
    bad = np.nonzero(gh != oh)[0]
    assert bad.size == 0, "%s: %d hit bits differ, first op %d (op %d key %d)" % (
        label, bad.size, bad[0], ops[bad[0]], keys[bad[0]])
    bad = np.nonzero(gv != ov)[0]
    assert bad.size == 0, "%s: %d values differ, first op %d (op %d key %d gpu %d oracle %d)" % (
        label, bad.size, bad[0], ops[bad[0]], keys[bad[0]], gv[bad[0]], ov[bad[0]])
    assert_same_contents(t, m, label)
    return gh


def _mixed(rng, n, key_pool, p=(0.5, 0.3, 0.2), vdtype=np.uint32):
    ops = rng.choice(np.array([0, 1, 2], np.uint8), size=n, p=list(p))
    keys = key_pool[rng.integers(0, key_pool.size, n)]
    vals = (rng.integers(1, 1 << 31, n)).astype(vdtype)
    return ops, keys, vals


def test_apply_unique_keys_u32():
    rng = np.random.default_rng(7)
    pool = unique_u32(1 << 20, seed=99)
    t = _dg().DyCuckoo(1 << 20)
    m = O.Map(1 << 20)
    # preload half, then a mixed batch over all keys, each key once
    pre = pool[: 1 << 19]
    t.insert(to_dev(pre), to_dev(pre ^ np.uint32(0x1234)))
    m.insert(pre, pre ^ np.uint32(0x1234))
    perm = rng.permutation(pool.size)
    keys = pool[perm]
    ops = rng.choice(np.array([0, 1, 2], np.uint8), size=keys.size)
    vals = rng.integers(1, 1 << 31, keys.size).astype(np.uint32)
    gh = _apply_and_compare(t, m, ops, keys, vals, "unique mixed")
    assert 0 < gh.sum() < keys.size
    t.close()


@pytest.mark.parametrize("distinct", [64, 5000, 300_000])
def test_apply_repeated_keys_u32(distinct):
    """Ops on few distinct keys: many ops per key in one batch; 64 distinct
    keys over 2^20 ops gives ~16k ops per key (the long-segment path)."""
    rng = np.random.default_rng(distinct)
    pool = unique_u32(distinct, seed=distinct + 1)
    t = _dg().DyCuckoo(1 << 16)
    m = O.Map()
    for b in range(3):
        ops, keys, vals = _mixed(rng, 1 << 20, pool)
        _apply_and_compare(t, m, ops, keys, vals, "repeated %d batch %d" % (distinct, b))
    t.close()


def test_apply_segment_length_boundaries():
    """Keys with exactly 63, 64, 65, 96 and 1000 ops in one batch, interleaved
    with keys seen once, covering both replay paths and their boundary."""
    rng = np.random.default_rng(3)
    heavy = unique_u32(5, seed=5)
    lengths = [63, 64, 65, 96, 1000]
    light = unique_u32(20000, seed=6)
    light = light[~np.isin(light, heavy)]
    keys = np.concatenate([np.repeat(heavy, lengths), light])
    keys = keys[rng.permutation(keys.size)]
    ops = rng.choice(np.array([0, 1, 2], np.uint8), size=keys.size, p=[0.4, 0.4, 0.2])
    vals = rng.integers(1, 1 << 31, keys.size).astype(np.uint32)
    t = _dg().DyCuckoo(1 << 16)
    m = O.Map()
    t.insert(to_dev(heavy[:3]), to_dev(heavy[:3]))
    m.insert(heavy[:3], heavy[:3])
    _apply_and_compare(t, m, ops, keys, vals, "segment boundaries")
    _apply_and_compare(t, m, ops, keys, vals + np.uint32(1), "segment boundaries again")
    t.close()


def test_apply_key_zero_and_unknown_ops():
    """Ops on key 0 miss and change nothing; op codes other than 0/1/2 read."""
    rng = np.random.default_rng(11)
    pool = np.concatenate([unique_u32(1000, seed=12), np.zeros(1, np.uint32)])
    ops, keys, vals = _mixed(rng, 100_000, pool)
    t = _dg().DyCuckoo(4096)
    m = O.Map()
    _apply_and_compare(t, m, ops, keys, vals, "key 0")
    ops2 = ops.copy()
    ops2[::7] = 9  # treated as find
    oracle_ops = ops2.copy()
    oracle_ops[oracle_ops > 2] = 0
    out, bits = t.apply(to_dev(ops2), to_dev(keys), to_dev(vals))
    ov, oh = m.apply(oracle_ops, keys.astype(np.uint64), vals.astype(np.uint64))
    assert np.array_equal(_dg().unpack_bits(bits, keys.size), oh)
    assert np.array_equal(to_host(out, 4).astype(np.uint64), ov)
    assert_same_contents(t, m, "unknown op codes")
    t.close()


@pytest.mark.parametrize("distinct", [100, 1 << 18])
def test_apply_u64_keys(distinct):
    rng = np.random.default_rng(distinct)
    pool = unique_u64(distinct, seed=77)
    t = _dg().DyCuckoo(1 << 16, key_bytes=8, value_bytes=8)
    m = O.Map()
    for b in range(2):
        ops, keys, vals = _mixed(rng, 1 << 19, pool, vdtype=np.uint64)
        vals = vals * np.uint64(0x100000001)
        _apply_and_compare(t, m, ops, keys, vals, "u64 %d batch %d" % (distinct, b))
    t.close()


def test_apply_spans_chunks_and_resizes():
    """A batch longer than one internal chunk (2^22 ops) keeps batch order
    across the chunk boundary; inserts grow the table, erases shrink it."""
    rng = np.random.default_rng(21)
    pool = unique_u32(1 << 21, seed=31)
    t = _dg().DyCuckoo(1 << 12)
    m = O.Map()
    n = (1 << 22) + 12345
    ops, keys, vals = _mixed(rng, n, pool, p=(0.2, 0.7, 0.1))
    _apply_and_compare(t, m, ops, keys, vals, "growth across chunks")
    cap_big = t.capacity
    # erase most keys: the post-batch policy may downsize
    present = m.export()[0].astype(np.uint32)
    er = present[rng.permutation(present.size)[: present.size * 9 // 10]]
    ops = np.full(er.size, 2, np.uint8)
    _apply_and_compare(t, m, ops, er, np.zeros(er.size, np.uint32), "mass erase")
    assert t.capacity <= cap_big
    t.close()


def test_resize_stream_u64_matches_oracle_every_batch():
    """The dynamic resize stream at reduced size: u64 keys and values, mixed
    batches that grow the table 2^11 -> 2^15 keys (60/30/10) and shrink it
    back (10/30/60), 5% in-batch repeats, upsize above 0.90 and downsize
    below 0.35 of capacity; every op result and the full contents equal the
    oracle after every batch, and the expected counts hold exactly."""
    from databases_gpu_gb300.workloads import ResizeStream
    ws = ResizeStream(batch_ops=1 << 14, grow=12, shrink=12, start=1 << 11, peak=1 << 15,
                      seed=10327)
    t = _dg().DyCuckoo(1 << 11, key_bytes=8, value_bytes=8, upper_load=0.90, lower_load=0.35,
                       min_downsize_capacity=0)
    m = O.Map()
    k0, v0 = ws.preload()
    t.insert(k0, v0)
    m.insert(k0.cpu().numpy().view(np.uint64), v0.cpu().numpy().view(np.uint64))
    peak_cap = 0
    ups = downs = 0
    for b in range(len(ws)):
        sb = ws.next()
        ops = sb.ops.cpu().numpy()
        keys = sb.keys.cpu().numpy().view(np.uint64)
        vals = sb.vals.cpu().numpy().view(np.uint64)
        gh = _apply_and_compare(t, m, ops, keys, vals, "stream batch %d (%s)" % (b, sb.phase))
        st = t.stats()
        ups += st["resizes_up"]
        downs += st["resizes_down"]
        assert t.size == sb.size_after
        assert int(gh[ops == 0].sum()) == sb.find_ops
        assert st["erased"] == sb.erase_hits
        assert t.size <= 0.90 * t.capacity + 1
        peak_cap = max(peak_cap, t.capacity)
    assert ups > 0 and downs > 0
    assert t.capacity < peak_cap
    t.close()


@pytest.mark.parametrize("flag", [True, False], ids=["flag", "detected"])
@pytest.mark.parametrize("key_bytes,bucket_bytes,chunk", [(4, 128, 0), (8, 128, 0), (4, 32, 0),
                                                         (8, 64, 4096)])
def test_apply_distinct_keys_one_pass_matches_oracle(key_bytes, bucket_bytes, chunk, flag):
    """Batches without key repeats take the one-pass path: with
    DYC_FLAG_UNIQUE by the caller's word, without it when the grouping meets
    no key twice (the path is picked on the device; chunks near the upsize
    bound take the general path). Five batches of distinct keys on a growing
    table: finds, upserts and erases of present keys, inserts of new keys
    (enough to fill buckets and need eviction walks and upsizes), erases and
    finds of absent keys, an op on key 0. Every op's value and hit bit and
    the contents after every batch equal the oracle's; with chunk, batches
    span many 4096-op chunks."""
    from databases_gpu_gb300 import _lib
    dg = _dg()
    L = _lib.lib()
    if chunk:
        assert L.dyc_debug_inject(_lib.INJECT_CHUNK_OPS, chunk) == 0
    try:
        t = dg.DyCuckoo(1 << 12, key_bytes=key_bytes, value_bytes=key_bytes,
                        bucket_bytes=bucket_bytes)
    finally:
        L.dyc_debug_inject(_lib.INJECT_RESET, 0)
    m = O.Map()
    rng = np.random.default_rng(83)
    pool = unique_u32(1 << 17, seed=84) if key_bytes == 4 else unique_u64(1 << 17, seed=84)
    npk = np.uint32 if key_bytes == 4 else np.uint64
    used = 0
    for r in range(5):
        present = m.export()[0].astype(npk)
        nold = min(present.size, 6000)
        old = rng.choice(present, nold, replace=False) if nold else np.zeros(0, npk)
        fresh = pool[used:used + 9000].astype(npk)
        used += 9000
        keys = np.concatenate([old[old != 0], fresh[fresh != 0], np.zeros(1, npk)])
        rng.shuffle(keys)
        n = keys.size
        ops = rng.choice(np.array([0, 1, 2], np.uint8), n, p=[0.3, 0.5, 0.2])
        vals = rng.integers(1, 1 << 30, n).astype(npk)
        _apply_and_compare(t, m, ops, keys, vals, "distinct batch %d" % r, unique=flag)
    assert len(m) > 15000 and t.capacity > (1 << 12)
    t.close()



@pytest.mark.parametrize("repeats", [False, True], ids=["distinct", "repeats"])
def test_apply_without_outputs(repeats):
    """dyc_apply with no value or bit output (both optional): a batch of
    distinct keys (the one-pass path) and one with repeats (the general
    path) leave the same contents as the oracle."""
    import ctypes as C
    import torch
    from databases_gpu_gb300 import _lib
    rng = np.random.default_rng(121)
    pool = unique_u32(1 << 16, seed=122)
    t = _dg().DyCuckoo(1 << 15)
    m = O.Map()
    t.insert(to_dev(pool[: 1 << 14]), to_dev(pool[: 1 << 14]))
    m.insert(pool[: 1 << 14], pool[: 1 << 14])
    n = 1 << 15
    keys = pool[rng.integers(0, pool.size, n)] if repeats else rng.permutation(pool)[:n]
    ops = rng.choice(np.array([0, 1, 2], np.uint8), n, p=[0.3, 0.5, 0.2])
    vals = rng.integers(1, 1 << 30, n).astype(np.uint32)
    dops, dkeys, dvals = to_dev(ops), to_dev(keys), to_dev(vals)
    L = _lib.lib()
    st = L.dyc_apply(t.handle, C.c_void_p(dops.data_ptr()), C.c_void_p(dkeys.data_ptr()),
                     C.c_void_p(dvals.data_ptr()), n, None, None, 0,
                     C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0
    torch.cuda.synchronize()
    m.apply(ops, keys.astype(np.uint64), vals.astype(np.uint64))
    assert_same_contents(t, m, "apply without outputs")
    t.close()
