"""GPU parity of table sets (dyc_set_apply): many tables served by one launch
sequence per batch.

Every table is compared, op by op and by full contents, with its own oracle
map after every round; the batched path, the per-table path
(dyc_set_apply_each) and the graph-replayed path give identical results.
Cases: tables of very different sizes, tables without ops in a round, small
tables hit by large batches (segments of up to kMidSeg ops per key and one
longer, sorted in chunks and merged), key 0, u64 keys, growth through the
per-table resize policy (before the inserts, or after the batch when it fits,
in waves over many tables), graph replay from fixed buffers at varying op
counts.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import assert_same_contents, to_host

pytestmark = pytest.mark.gpu


def _dg():
    import databases_gpu_gb300 as dg
    return dg


def _check_round(S, maps, w_off, ops, keys, vals, out, bits, label):
    n = keys.numel()
    gv = to_host(out, S.value_bytes).astype(np.uint64)
    gh = _dg().unpack_bits(bits, n)
    o = ops.cpu().numpy()
    kb = S.key_bytes
    k = to_host(keys, kb).astype(np.uint64)
    v = to_host(vals, S.value_bytes).astype(np.uint64)
    for t in range(S.ntables):
        a, b = int(w_off[t]), int(w_off[t + 1])
        if a == b:
            continue
        ov, oh = maps[t].apply(o[a:b], k[a:b], v[a:b])
        assert np.array_equal(gh[a:b], oh), "%s: table %d hit bits differ" % (label, t)
        assert np.array_equal(gv[a:b], ov), "%s: table %d values differ" % (label, t)
    sizes, caps = S.sizes()
    for t in range(S.ntables):
        assert int(sizes[t]) == len(maps[t]), "%s: table %d size" % (label, t)
        assert sizes[t] <= caps[t]


def _small_workload(ntables, seed, log2_size=(2, 12), log2_batch=(0, 13)):
    from databases_gpu_gb300.workloads import MultiTableWorkload
    return MultiTableWorkload(ntables, log2_size=log2_size, log2_batch=log2_batch, seed=seed)


def _preload(S, w, maps):
    for t in range(S.ntables):
        k, v = w.preload(t)
        S.table(t).insert(k, v)
        maps[t].insert(to_host(k, 4), to_host(v, 4))


@pytest.mark.parametrize("graph,tuned,l2", [(False, False, 0), (True, False, 0), (False, True, 0),
                                              (False, False, 2)])
def test_set_matches_oracle_per_table(graph, tuned, l2):
    """tuned: per-table subtable counts and eviction bounds (2..4, 1..256, as
    a tuner may pick), 64-byte buckets and a launch cap of 2 blocks per SM.
    l2 = 2: the members' probes carry L2 eviction-priority hints."""
    w = _small_workload(96, seed=5)
    if l2:
        S = _dg().DyCuckooSet(w.sizes.numpy(), max_evictions=64, l2_resident=l2)
    elif tuned:
        rng = np.random.default_rng(2)
        S = _dg().DyCuckooSet(w.sizes.numpy(), bucket_bytes=64,
                              num_subtables=rng.integers(2, 5, 96))
        S.configure(2, rng.choice(np.array([1, 16, 256], np.uint32), 96))
    else:
        S = _dg().DyCuckooSet(w.sizes.numpy(), max_evictions=64)
    maps = [O.Map() for _ in range(S.ntables)]
    _preload(S, w, maps)
    for r in range(4):
        ops, keys, vals = w.round()
        out, bits = S.apply(w.offsets, ops, keys, vals, h_offsets=w.offsets_host, graph=graph)
        _check_round(S, maps, w.offsets_host, ops, keys, vals, out, bits, "round %d" % r)
    for t in (0, 17, 95):
        assert_same_contents(S.table(t), maps[t], "table %d contents" % t)
    S.close()


def test_set_batched_equals_per_table_path():
    w = _small_workload(128, seed=9)
    A = _dg().DyCuckooSet(w.sizes.numpy())
    B = _dg().DyCuckooSet(w.sizes.numpy())
    for t in range(A.ntables):
        k, v = w.preload(t)
        A.table(t).insert(k, v)
        B.table(t).insert(k, v)
    for r in range(3):
        ops, keys, vals = w.round()
        oa, ba = A.apply(w.offsets, ops, keys, vals, h_offsets=w.offsets_host)
        ob, bb = B.apply(w.offsets, ops, keys, vals, h_offsets=w.offsets_host, each=True)
        assert bool((oa == ob).all()), "round %d: values differ" % r
        assert bool((ba == bb).all()), "round %d: bits differ" % r
        sa, _ = A.sizes()
        sb, _ = B.sizes()
        assert np.array_equal(sa, sb)
    for t in range(0, A.ntables, 7):
        ka, va = A.table(t).export()
        kb_, vb_ = B.table(t).export()
        assert bool((ka == kb_).all()) and bool((va == vb_).all())
    A.close()
    B.close()


def test_set_long_segments_key_zero_and_empty_tables():
    """Table 0: a few keys hit thousands of times (mid segments) and one key
    hit 6000 times (longer than one shared-memory sort); table 1 has no ops;
    table 2 gets key 0."""
    import torch
    rng = np.random.default_rng(4)
    S = _dg().DyCuckooSet([64, 1000, 5000])
    maps = [O.Map() for _ in range(3)]
    hot = rng.integers(1, 1 << 31, 40).astype(np.uint32)
    k0 = np.concatenate([np.repeat(hot[:1], 6000), hot[rng.integers(1, 40, 20000)]])
    k0 = k0[rng.permutation(k0.size)]
    k2 = rng.integers(0, 3, 3000).astype(np.uint32)  # keys 0, 1 and 2
    keys = np.concatenate([k0, k2])
    ops = rng.choice(np.array([0, 1, 2], np.uint8), size=keys.size, p=[0.4, 0.4, 0.2])
    vals = rng.integers(1, 1 << 31, keys.size).astype(np.uint32)
    off = np.array([0, k0.size, k0.size, keys.size], np.uint32)
    d = lambda a: torch.from_numpy(a.view(np.int32) if a.dtype == np.uint32 else a).cuda()
    for r in range(2):
        out, bits = S.apply(d(off), d(ops), d(keys), d(vals + np.uint32(r)), h_offsets=off)
        _check_round(S, maps, off, d(ops), d(keys), d(vals + np.uint32(r)), out, bits,
                     "long segments round %d" % r)
    S.close()


def test_set_u64_keys_and_growth():
    """u64 keys / u64 values; tables start tiny and grow through the per-table
    upsize policy inside the set call."""
    import torch
    rng = np.random.default_rng(8)
    nt = 40
    S = _dg().DyCuckooSet([16] * nt, key_bytes=8, value_bytes=8)
    maps = [O.Map() for _ in range(nt)]
    for r in range(3):
        cnt = rng.integers(0, 3000, nt)
        off = np.zeros(nt + 1, np.uint32)
        off[1:] = np.cumsum(cnt)
        n = int(off[-1])
        keys = rng.integers(1, 1 << 62, n, dtype=np.int64).astype(np.uint64) % np.uint64(5000) + \
            np.uint64(1 << 40)
        ops = rng.choice(np.array([0, 1, 2], np.uint8), size=n, p=[0.3, 0.6, 0.1])
        vals = rng.integers(0, 1 << 62, n, dtype=np.int64).astype(np.uint64)
        dk = torch.from_numpy(keys.view(np.int64)).cuda()
        dv = torch.from_numpy(vals.view(np.int64)).cuda()
        do = torch.from_numpy(ops).cuda()
        doff = torch.from_numpy(off.view(np.int32)).cuda()
        out, bits = S.apply(doff, do, dk, dv, h_offsets=off)
        _check_round(S, maps, off, do, dk, dv, out, bits, "u64 round %d" % r)
    st = S.stats()
    sizes, caps = S.sizes()
    assert caps.max() > 16 * 4  # tables grew
    S.close()


@pytest.mark.parametrize("key_bytes", [4, 8])
def test_set_rounds_of_mostly_single_op_keys(key_bytes):
    """Rounds in which most keys have one op (resolved by the one-pass
    kernel in phase B) and some tables have repeats (through the per-key
    passes), in the same round: per table, distinct keys for finds, upserts
    and erases of present keys, inserts of new keys that fill buckets and
    need eviction walks and upsizes, finds and erases of absent keys, and
    key 0; every third table also repeats a few of its keys. Every op's
    value and bit and every table's size equal its oracle's."""
    import torch
    rng = np.random.default_rng(71 + key_bytes)
    nt = 64
    sizes = np.round(2.0 ** (6 + 6 * rng.random(nt))).astype(np.int64)
    S = _dg().DyCuckooSet(sizes, key_bytes=key_bytes, value_bytes=key_bytes)
    maps = [O.Map() for _ in range(nt)]
    npk, tdt = (np.uint32, np.int32) if key_bytes == 4 else (np.uint64, np.int64)
    top = (1 << 31) if key_bytes == 4 else (1 << 62)
    for r in range(4):
        parts = []
        for t in range(nt):
            present = maps[t].export()[0].astype(npk)
            m = int(rng.integers(0, 2 * sizes[t] + 2))
            old = rng.choice(present, min(present.size, m // 3), replace=False) \
                if present.size else np.zeros(0, npk)
            new = np.unique(rng.integers(1, top, m - old.size, dtype=np.int64).astype(npk))
            k = np.concatenate([old, new])
            k = k[~np.isin(k, np.zeros(1, npk))]
            if t % 3 == 0 and k.size:  # a few repeats in this table
                k = np.concatenate([k, rng.choice(k, min(k.size, 5))])
            if t % 5 == 0:
                k = np.concatenate([k, np.zeros(1, npk)])  # key 0
            parts.append(k[rng.permutation(k.size)])
        off = np.zeros(nt + 1, np.uint32)
        off[1:] = np.cumsum([p.size for p in parts])
        keys = np.concatenate(parts).astype(npk)
        n = keys.size
        ops = rng.choice(np.array([0, 1, 2], np.uint8), size=n, p=[0.35, 0.45, 0.2])
        vals = rng.integers(1, top, n, dtype=np.int64).astype(npk)
        dk = torch.from_numpy(keys.view(tdt)).cuda()
        dv = torch.from_numpy(vals.view(tdt)).cuda()
        do = torch.from_numpy(ops).cuda()
        doff = torch.from_numpy(off.view(np.int32)).cuda()
        out, bits = S.apply(doff, do, dk, dv, h_offsets=off, graph=(r % 2 == 1))
        _check_round(S, maps, off, do, dk, dv, out, bits, "single-op round %d" % r)
    for t in range(nt):
        assert_same_contents(S.table(t), maps[t], "table %d after the rounds" % t)
    S.close()


def test_tuner_picks_a_measured_candidate():
    from databases_gpu_gb300 import tune
    space = {"bucket_bytes": (64, 128), "num_subtables": (2, 4), "max_evictions": (16, 64)}
    r = tune.tune_class(10, 512, space, rounds=2)
    assert len(r.candidates) == 8
    assert r.best in [{k: c[k] for k in ("bucket_bytes", "num_subtables", "max_evictions")}
                      for c in r.candidates]
    assert r.mops > 0 and set(r.by_bucket) == {64, 128}
    sb, d, ev = tune.plan_set([1000, 1100], [500, 600], {9: r, 10: r})
    assert sb in (64, 128) and list(d) == [r.by_bucket[sb][0]["num_subtables"]] * 2


def test_set_graph_reuses_buffers_across_batch_sizes():
    """Fixed staging buffers (as a request server holds them), a different op
    count every round: the captured graphs read the count on the device, so
    each round replays the same graph. Rounds that cannot grow a table run
    both phases back to back; the growing rounds (small tables, many inserts)
    take the path with an upsize between the phases, also under the graph.
    Two rounds skip the resize policy (a different captured sequence for the
    same buffers). Capacities follow a twin set fed the same rounds through
    one dyc_apply per table."""
    import torch
    rng = np.random.default_rng(13)
    nt = 48
    sizes = rng.integers(64, 4096, nt).tolist()
    S = _dg().DyCuckooSet(sizes)
    twin = _dg().DyCuckooSet(sizes)
    maps = [O.Map() for _ in range(nt)]
    cap = nt * 2500
    b_ops = torch.empty(cap, dtype=torch.uint8, device="cuda")
    b_keys = torch.empty(cap, dtype=torch.int32, device="cuda")
    b_vals = torch.empty(cap, dtype=torch.int32, device="cuda")
    b_out = torch.empty(cap, dtype=torch.int32, device="cuda")
    b_bits = torch.empty(cap // 32 + 1, dtype=torch.int32, device="cuda")
    b_off = torch.empty(nt + 1, dtype=torch.int32, device="cuda")
    for r in range(8):
        grow = r in (2, 5)
        cnt = rng.integers(0, 2500 if grow else 600, nt)
        off = np.zeros(nt + 1, np.uint32)
        off[1:] = np.cumsum(cnt)
        n = int(off[-1])
        p = [0.1, 0.85, 0.05] if grow else [0.6, 0.2, 0.2]
        ops = rng.choice(np.array([0, 1, 2], np.uint8), size=n, p=p)
        keys = rng.integers(1, 1 << 20, n).astype(np.uint32)
        vals = rng.integers(0, 1 << 31, n).astype(np.uint32)
        b_ops[:n].copy_(torch.from_numpy(ops))
        b_keys[:n].copy_(torch.from_numpy(keys.view(np.int32)))
        b_vals[:n].copy_(torch.from_numpy(vals.view(np.int32)))
        b_off.copy_(torch.from_numpy(off.view(np.int32)))
        nw = (n + 31) // 32
        fixed = r in (3, 6)
        out, bits = S.apply(b_off, b_ops[:n], b_keys[:n], b_vals[:n], out=b_out[:n],
                            bits=b_bits[:nw], h_offsets=off, graph=True, no_resize=fixed)
        _check_round(S, maps, off, b_ops[:n], b_keys[:n], b_vals[:n], out, bits,
                     "graph round %d (n=%d)" % (r, n))
        twin.apply(b_off, b_ops[:n], b_keys[:n], b_vals[:n], h_offsets=off, each=True,
                   no_resize=fixed)
        assert np.array_equal(S.sizes()[1], twin.sizes()[1]), "round %d capacities" % r
    for t in (0, 21, nt - 1):
        assert_same_contents(S.table(t), maps[t], "table %d contents" % t)
    S.close()
    twin.close()


@pytest.mark.parametrize("kind", ["new_keys", "half_updates"])
@pytest.mark.parametrize("device_upsize", [0, 1])
def test_set_deferred_upsize_matches_per_table_path(kind, device_upsize):
    """new_keys: tables preloaded to 70 % of their slots (below the 0.8 upper
    bound), then a batch of new keys worth 15 % more. half_updates: preloaded
    to 70 %, a batch worth 16 % of which half update present keys, so only
    counting every insert (as the reference's policy does) passes the bound.
    One upsize per table brings each back under the bound. With upsize
    targets kept ahead (device_upsize 0) the policy runs on the device
    between the phases; without them (1) either batch keeps the tables within
    90 % (halfway from the bound to full) even if all its ops were new keys,
    so the set runs it without a host round trip and applies the upsize
    policy afterwards (entries the fuller tables could not place take the
    overflow path). Either way results, sizes, capacities and contents equal
    those of one dyc_apply per table, which upsizes before inserting."""
    import torch
    rng = np.random.default_rng(21)
    nt = 8
    A = _dg().DyCuckooSet([3000] * nt, device_upsize=device_upsize)
    B = _dg().DyCuckooSet([3000] * nt)
    _, caps = A.sizes()
    maps = [O.Map() for _ in range(nt)]
    pre = 0.70
    share = 0.15 if kind == "new_keys" else 0.16
    preloaded = []
    for t in range(nt):
        m = int(pre * int(caps[t]))
        k = (np.arange(m, dtype=np.uint64) * 2654435761 % (1 << 31) + 1).astype(np.uint32)
        k = np.unique(k)
        v = rng.integers(0, 1 << 31, k.size).astype(np.uint32)
        dk = torch.from_numpy(k.view(np.int32)).cuda()
        dv = torch.from_numpy(v.view(np.int32)).cuda()
        A.table(t).insert(dk, dv)
        B.table(t).insert(dk, dv)
        maps[t].insert(k, v)
        preloaded.append(k)
    assert np.array_equal(A.sizes()[1], caps)  # no upsize while preloading
    cnt = (share * caps.astype(np.float64)).astype(np.int64)
    off = np.zeros(nt + 1, np.uint32)
    off[1:] = np.cumsum(cnt)
    n = int(off[-1])
    keys = rng.integers((1 << 31) + 1, (1 << 32) - 1, n, dtype=np.uint64).astype(np.uint32)
    if kind == "half_updates":
        for t in range(nt):
            a, h = int(off[t]), int(cnt[t]) // 2
            keys[a:a + h] = rng.choice(preloaded[t], h, replace=False)
    ops = np.ones(n, np.uint8)
    vals = rng.integers(0, 1 << 31, n).astype(np.uint32)
    d = lambda a: torch.from_numpy(a.view(np.int32) if a.dtype == np.uint32 else a).cuda()
    oa, ba = A.apply(d(off), d(ops), d(keys), d(vals), h_offsets=off)
    sa = A.stats()
    ob, bb = B.apply(d(off), d(ops), d(keys), d(vals), h_offsets=off, each=True)
    _check_round(A, maps, off, d(ops), d(keys), d(vals), oa, ba, "deferred upsize")
    assert bool((oa == ob).all()) and bool((ba == bb).all())
    sza, capa = A.sizes()
    szb, capb = B.sizes()
    assert np.array_equal(sza, szb)
    assert np.array_equal(capa, capb), (capa, capb)
    assert sa["resizes_up"] >= nt
    assert sa["split_phases"] == 0  # no host read between the phases
    for t in range(nt):
        assert_same_contents(A.table(t), maps[t], "table %d contents" % t)
    A.close()
    B.close()


@pytest.mark.parametrize("bucket_bytes,key_bytes", [(128, 4), (64, 8)])
@pytest.mark.parametrize("device_upsize", [0, 1])
def test_set_upsize_waves_match_per_table_path(bucket_bytes, key_bytes, device_upsize):
    """Many tiny tables, each hit by enough inserts to need several upsizes in
    one batch: the set issues them in waves (one launch per wave for all its
    tables; with upsize targets kept ahead the device makes the first upsize
    of each table and the host the rest). Capacities, sizes, results and
    contents equal those of one dyc_apply per table, which upsizes table by
    table."""
    import torch
    rng = np.random.default_rng(23)
    nt = 200
    A = _dg().DyCuckooSet([64] * nt, key_bytes=key_bytes, bucket_bytes=bucket_bytes,
                          device_upsize=device_upsize)
    B = _dg().DyCuckooSet([64] * nt, key_bytes=key_bytes, bucket_bytes=bucket_bytes)
    maps = [O.Map() for _ in range(nt)]
    for r in range(2):
        cnt = rng.integers(0, 2000, nt)
        off = np.zeros(nt + 1, np.uint32)
        off[1:] = np.cumsum(cnt)
        n = int(off[-1])
        ops = rng.choice(np.array([0, 1, 2], np.uint8), size=n, p=[0.1, 0.8, 0.1])
        if key_bytes == 4:
            keys = rng.integers(1, 1 << 31, n).astype(np.uint32)
            vals = rng.integers(0, 1 << 31, n).astype(np.uint32)
            dk = torch.from_numpy(keys.view(np.int32)).cuda()
            dv = torch.from_numpy(vals.view(np.int32)).cuda()
        else:
            keys = rng.integers(1, 1 << 62, n, dtype=np.int64).astype(np.uint64)
            vals = rng.integers(0, 1 << 62, n, dtype=np.int64).astype(np.uint64)
            dk = torch.from_numpy(keys.view(np.int64)).cuda()
            dv = torch.from_numpy(vals.view(np.int64)).cuda()
        do = torch.from_numpy(ops).cuda()
        doff = torch.from_numpy(off.view(np.int32)).cuda()
        oa, ba = A.apply(doff, do, dk, dv, h_offsets=off, graph=(r == 1))
        st = A.stats()
        ob, bb = B.apply(doff, do, dk, dv, h_offsets=off, each=True)
        _check_round(A, maps, off, do, dk, dv, oa, ba, "waves round %d" % r)
        assert bool((oa == ob).all()) and bool((ba == bb).all())
        sza, capa = A.sizes()
        szb, capb = B.sizes()
        assert np.array_equal(sza, szb) and np.array_equal(capa, capb)
        assert st["resizes_up"] > 2 * nt  # several upsizes per table
    for t in (0, 99, nt - 1):
        assert_same_contents(A.table(t), maps[t], "table %d contents" % t)
    A.close()
    B.close()


@pytest.mark.parametrize("keep", [True, False], ids=["spare_cache", "no_cache"])
@pytest.mark.parametrize("key_bytes", [4, 8])
def test_set_device_upsize_policy_matches_host_policy(key_bytes, keep):
    """Tables of 2^5..2^9 keys preloaded near the 0.8 bound take six rounds
    of mixed batches (from fixed buffers: the later rounds replay captured
    graphs) that
    make many of them grow: a set that keeps an upsize target ahead for every
    member (the policy on the device, between the phases) and one that
    applies the policy on the host between the phases give the same results,
    sizes, capacities and contents, equal to the oracle's. Rounds in which
    every growing table needs one upsize run with no host read between the
    phases; the spare targets are counted by dyc_set_spare_bytes. With the
    spare cache (the default) replaced subtables serve as later spares;
    without it (dyc_set_spare_cache 0) every spare is a fresh allocation."""
    import torch
    rng = np.random.default_rng(41)
    nt = 300
    sizes = np.round(2.0 ** (5 + 4 * rng.random(nt))).astype(np.int64)
    kw = dict(key_bytes=key_bytes, value_bytes=key_bytes)
    A = _dg().DyCuckooSet(sizes, device_upsize=0, **kw)
    if not keep:
        A.spare_cache(0)
    B = _dg().DyCuckooSet(sizes, device_upsize=1, **kw)
    maps = [O.Map() for _ in range(nt)]
    npk, tdt = (np.uint32, np.int32) if key_bytes == 4 else (np.uint64, np.int64)
    top = (1 << 31) if key_bytes == 4 else (1 << 62)
    live = []
    for t in range(nt):
        k = np.unique(rng.integers(1, top, int(0.78 * sizes[t]) + 1, dtype=np.int64)).astype(npk)
        v = rng.integers(0, top, k.size, dtype=np.int64).astype(npk)
        dk = torch.from_numpy(k.view(tdt)).cuda()
        dv = torch.from_numpy(v.view(tdt)).cuda()
        A.table(t).insert(dk, dv)
        B.table(t).insert(dk, dv)
        maps[t].insert(k.astype(np.uint64), v.astype(np.uint64))
        live.append(k)
    # fixed buffers (rounds 2.. replay the captured graphs of each set)
    cap = int(2 * (sizes // 8).sum()) + 32
    tt = torch.int32 if key_bytes == 4 else torch.int64
    b_ops = torch.empty(cap, dtype=torch.uint8, device="cuda")
    b_keys = torch.empty(cap, dtype=tt, device="cuda")
    b_vals = torch.empty(cap, dtype=tt, device="cuda")
    b_off = torch.empty(nt + 1, dtype=torch.int32, device="cuda")
    outs = [(torch.empty(cap, dtype=tt, device="cuda"),
             torch.empty(cap // 32 + 1, dtype=torch.int32, device="cuda")) for _ in range(2)]
    device_rounds = 0
    for r in range(6):
        cnt = rng.integers(0, 3, nt) * (sizes // 8)
        off = np.zeros(nt + 1, np.uint32)
        off[1:] = np.cumsum(cnt)
        n = int(off[-1])
        ops = rng.choice(np.array([0, 1, 2], np.uint8), size=n, p=[0.3, 0.6, 0.1])
        keys = rng.integers(1, top, n, dtype=np.int64).astype(npk)
        for t in range(nt):  # a third of each table's ops on its present keys
            a, b = int(off[t]), int(off[t + 1])
            m = (b - a) // 3
            if m:
                keys[a:a + m] = rng.choice(live[t], m)
        vals = rng.integers(0, top, n, dtype=np.int64).astype(npk)
        b_ops[:n].copy_(torch.from_numpy(ops))
        b_keys[:n].copy_(torch.from_numpy(keys.view(tdt)))
        b_vals[:n].copy_(torch.from_numpy(vals.view(tdt)))
        b_off.copy_(torch.from_numpy(off.view(np.int32)))
        do, dk, dv, nw = b_ops[:n], b_keys[:n], b_vals[:n], (n + 31) // 32
        oa, ba = A.apply(b_off, do, dk, dv, out=outs[0][0][:n], bits=outs[0][1][:nw],
                         h_offsets=off, graph=True)
        sa = A.stats()
        ob, bb = B.apply(b_off, do, dk, dv, out=outs[1][0][:n], bits=outs[1][1][:nw],
                         h_offsets=off, graph=True)
        _check_round(A, maps, off, do, dk, dv, oa, ba, "round %d" % r)
        assert bool((oa == ob).all()) and bool((ba == bb).all()), "round %d" % r
        sza, capa = A.sizes()
        szb, capb = B.sizes()
        assert np.array_equal(sza, szb) and np.array_equal(capa, capb), "round %d" % r
        if sa["resizes_up"] > 0 and sa["split_phases"] == 0:
            device_rounds += 1
        for t in range(nt):
            a, b = int(off[t]), int(off[t + 1])
            ins = keys[a:b][ops[a:b] == 1]
            if ins.size:
                live[t] = np.union1d(live[t], ins)
    assert device_rounds >= 2, device_rounds
    assert A.spare_bytes() > 0 and B.spare_bytes() == 0
    for t in range(0, nt, 23):
        assert_same_contents(A.table(t), maps[t], "table %d contents" % t)
    A.close()
    B.close()


@pytest.mark.parametrize("graph", [False, True])
def test_set_device_offsets_disagreeing_with_host_offsets_are_reported(graph):
    """The kernels read a set batch's op count and table ranges from the
    device offsets, while the host sized everything from h_offsets. Device
    offsets whose total is larger than the host's, or that are out of order,
    are clamped by the kernels (every access stays inside the batch's
    buffers) and the call returns DYC_EINVAL. With only the total too large
    the batch is still applied exactly as the host's offsets describe it.
    Under graph replay all calls use the same buffers, so the second and
    third calls replay the captured graph with the offsets changed in place."""
    import torch
    from databases_gpu_gb300._lib import DYC_EINVAL
    dg = _dg()
    w = _small_workload(16, seed=11, log2_size=(4, 10), log2_batch=(4, 9))
    S = dg.DyCuckooSet(w.sizes.numpy(), max_evictions=64)
    maps = [O.Map() for _ in range(S.ntables)]
    _preload(S, w, maps)
    h_off = w.offsets_host
    n = int(h_off[-1])
    d_off = torch.empty(S.ntables + 1, dtype=torch.int32, device="cuda")
    b_ops = torch.empty(n, dtype=torch.uint8, device="cuda")
    b_keys = torch.empty(n, dtype=torch.int32, device="cuda")
    b_vals = torch.empty(n, dtype=torch.int32, device="cuda")
    out = torch.empty(n, dtype=torch.int32, device="cuda")
    bits = torch.empty((n + 31) // 32, dtype=torch.int32, device="cuda")

    def run(offsets):
        ops, keys, vals = w.round()
        b_ops.copy_(ops)
        b_keys.copy_(keys)
        b_vals.copy_(vals)
        d_off.copy_(torch.from_numpy(np.asarray(offsets, np.int64).astype(np.uint32)
                                     .view(np.int32)))
        S.apply(d_off, b_ops, b_keys, b_vals, out=out, bits=bits, h_offsets=h_off, graph=graph)
        return ops, keys, vals

    # a clean round (warms the graph entry for these buffers)
    ops, keys, vals = run(h_off)
    _check_round(S, maps, h_off, ops, keys, vals, out, bits, "clean")
    # the device total exceeds the host's op count: clamped to it, reported
    big = h_off.astype(np.int64).copy()
    big[-1] = n + 100
    with pytest.raises(dg.DycError) as ei:
        run(big)
    assert ei.value.status == DYC_EINVAL, ei.value
    o = b_ops.cpu().numpy()
    k = to_host(b_keys, 4).astype(np.uint64)
    v = to_host(b_vals, 4).astype(np.uint64)
    for t in range(S.ntables):
        a, b = int(h_off[t]), int(h_off[t + 1])
        maps[t].apply(o[a:b], k[a:b], v[a:b])
    for t in range(S.ntables):
        assert_same_contents(S.table(t), maps[t], "table %d after the clamped round" % t)
    # offsets out of order with the right total: reported (the tables got
    # ops under the wrong ranges, so their contents are not checked)
    bad = h_off.astype(np.int64).copy()
    bad[1], bad[2] = bad[2], bad[1]
    if bad[1] == bad[2]:
        bad[1] = bad[2] + 1
    with pytest.raises(dg.DycError) as ei:
        run(bad)
    assert ei.value.status == DYC_EINVAL, ei.value
    torch.cuda.synchronize()
    S.close()
