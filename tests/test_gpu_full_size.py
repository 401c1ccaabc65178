"""Parity at full size for the resize stream, the 4096-table set and the
serving loop, against the oracle.

The oracle map cannot follow billions of operations in a test, but a key's
results depend only on that key's own operations, in batch order. So each
test fixes a class of keys by a bit pattern of the key (1/16 or 1/64 of all
keys), runs the full-size workload on the GPU, and hands every operation on a
key of that class, in its original order, to the oracle: the GPU's result of
each such operation (value and hit bit) must equal the oracle's, and the
table's entries of that class must equal the oracle map's contents. Every
batch, table and tenant of the workload takes part; only the keys checked are
a sample.
"""
import ctypes as C
import threading

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _dg():
    import databases_gpu_gb300 as dg
    return dg


def _u64(t):
    return t.cpu().numpy().view(np.uint64)


def _u32(t):
    return t.cpu().numpy().view(np.uint32)


def _export_class(table, mask_fn, torch):
    """The table's entries whose keys pass mask_fn, as sorted host arrays
    (dyc_export into device buffers, filtered on the device)."""
    L = _dg().lib()
    cap = max(table.size, 1)
    kd = torch.empty(cap, dtype=table.key_dtype(), device="cuda")
    vd = torch.empty(cap, dtype=table.value_dtype(), device="cuda")
    got = C.c_uint64()
    rc = L.dyc_export(table.handle, C.c_void_p(kd.data_ptr()), C.c_void_p(vd.data_ptr()), cap,
                      C.byref(got), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, L.dyc_last_error()
    m = int(got.value)
    assert m == table.size, (m, table.size)
    kd, vd = kd[:m], vd[:m]
    sel = mask_fn(kd)
    k = kd[sel].cpu().numpy().view(np.uint64 if table.key_bytes == 8 else np.uint32)
    v = vd[sel].cpu().numpy().view(np.uint64 if table.value_bytes == 8 else np.uint32)
    order = np.argsort(k, kind="stable")
    return k[order].astype(np.uint64), v[order].astype(np.uint64)


def _same_contents(k, v, omap, label):
    ok_, ov_ = omap.export()
    assert k.size == ok_.size, "%s: %d entries vs %d in the oracle" % (label, k.size, ok_.size)
    assert np.array_equal(k, ok_), "%s: key sets differ" % label
    assert np.array_equal(v, ov_), "%s: %d values differ" % (label, int((v != ov_).sum()))


def test_resize_stream_full_size_on_a_key_class():
    """The full dynamic resize stream: u64 keys / values, 512 batches of 2^22
    mixed ops growing the table from 2^20 to 2^27 keys and shrinking it back
    (upsize above 0.90, downsize below 0.35, 5 % in-batch repeats), through
    dyc_apply. Keys with their low 6 bits clear (1/64) are followed by the
    oracle: every such op's result, every batch, and the class's contents
    after every 16th batch and after every batch that resized."""
    import torch
    dg = _dg()
    from databases_gpu_gb300.workloads import ResizeStream
    dev = torch.device("cuda", 0)
    B = 1 << 22
    ws = ResizeStream(B, 256, 256, 1 << 20, 1 << 27, dup=0.05, seed=10327, device=dev)
    t = dg.DyCuckoo(1 << 20, key_bytes=8, value_bytes=8, upper_load=0.90, lower_load=0.35,
                    min_downsize_capacity=0, max_evictions=2048)
    dg.pool_reserve(4 << 30)

    def in_class(k):
        return (k & 63) == 0

    omap = O.Map(1 << 22)
    k0, v0 = ws.preload()
    t.insert(k0, v0)
    s0 = in_class(k0)
    omap.insert(_u64(k0[s0]), _u64(v0[s0]))
    del k0, v0
    out = torch.empty(B, dtype=torch.int64, device=dev)
    bits = torch.empty((B + 31) // 32, dtype=torch.int32, device=dev)
    sh = torch.arange(32, dtype=torch.int32, device=dev)
    checked_ops = checkpoints = resizes = 0
    for b in range(len(ws)):
        sb = ws.next()
        t.apply(sb.ops, sb.keys, sb.vals, out=out, bits=bits)
        st = t.stats()
        sel = torch.nonzero(in_class(sb.keys)).flatten()
        hits = ((bits.view(-1, 1) >> sh) & 1).flatten()[:B].bool()
        ov, oh = omap.apply(sb.ops[sel].cpu().numpy(), _u64(sb.keys[sel]), _u64(sb.vals[sel]))
        gv, gh = _u64(out[sel]), hits[sel].cpu().numpy()
        assert np.array_equal(gh, oh), "batch %d: %d hit bits differ" % (b, int((gh != oh).sum()))
        assert np.array_equal(gv, ov), "batch %d: %d values differ" % (b, int((gv != ov).sum()))
        checked_ops += int(sel.numel())
        assert t.size == sb.size_after, (b, t.size, sb.size_after)
        resized = st["resizes_up"] + st["resizes_down"]
        resizes += resized
        if resized or b % 16 == 15:
            k, v = _export_class(t, in_class, torch)
            _same_contents(k, v, omap, "after batch %d" % b)
            checkpoints += 1
    assert resizes >= 40 and checkpoints >= 32 and checked_ops > 2.5e7, (
        resizes, checkpoints, checked_ops)
    t.close()


def test_multi_table_set_full_size_on_a_key_class():
    """The 4096-table workload at full size (tables of 2^8..2^20 keys, about
    5.1e8 keys, 3.35e7 mixed ops per round), three rounds through the set's
    graph path. Keys with their low 4 bits clear (1/16) are followed
    by one oracle map per table: every such op's result and, after the
    rounds, every table's entries of the class."""
    import torch
    dg = _dg()
    from databases_gpu_gb300.workloads import MultiTableWorkload
    w = MultiTableWorkload(4096, seed=10327, device="cuda")
    S = dg.DyCuckooSet(w.sizes.numpy())

    def in_class(k):
        return (k & 15) == 0

    maps = [O.Map() for _ in range(w.ntables)]
    for i in range(w.ntables):
        k, v = w.preload(i)
        S.table(i).insert(k, v, new_keys=True, unique=True)
        s = in_class(k)
        maps[i].insert(_u32(k[s]), _u32(v[s]))
    off = w.offsets_host.astype(np.int64)
    n = int(off[-1])
    out = torch.empty(n, dtype=torch.int32, device="cuda")
    bits = torch.empty((n + 31) // 32, dtype=torch.int32, device="cuda")
    checked = 0
    for r in range(3):
        ops, keys, vals = w.round()
        S.apply(w.offsets, ops, keys, vals, out=out, bits=bits, h_offsets=w.offsets_host,
                graph=True)
        sel = torch.nonzero(in_class(keys)).flatten()
        si = sel.cpu().numpy()
        hits = _dg().unpack_bits(bits, n)[si]
        gv = _u32(out[sel])
        o, k, v = ops[sel].cpu().numpy(), _u32(keys[sel]), _u32(vals[sel])
        tab = np.searchsorted(off, si, side="right") - 1
        for i in np.unique(tab):
            m = tab == i
            ov, oh = maps[i].apply(o[m], k[m].astype(np.uint64), v[m].astype(np.uint64))
            assert np.array_equal(hits[m], oh), "round %d table %d: hit bits differ" % (r, i)
            assert np.array_equal(gv[m].astype(np.uint64), ov), \
                "round %d table %d: values differ" % (r, i)
        checked += si.size
    for i in range(w.ntables):
        kk, vv = _export_class(S.table(i), in_class, torch)
        _same_contents(kk, vv, maps[i], "table %d" % i)
    assert checked > 5e6, checked
    S.close()


def test_serving_full_size_on_a_key_class():
    """The serving loop's tenants at full size: 64 u64/u32 tables of
    2^16..2^24 keys (about 2e8 keys preloaded), 3000 requests of log-uniform
    32..65536 ops (70 % find / 20 % insert / 10 % erase) on Zipf(0.9)
    tenants, submitted from four threads and coalesced into shared steps by
    the server (continuous batching) under a 120 GB admission cap. Keys with
    their low 6 bits clear are followed by one oracle map per tenant, fed each
    tenant's requests in submission order: every such op's result and, at
    the end, every tenant's entries of the class."""
    import torch
    dg = _dg()
    from databases_gpu_gb300.workloads import splitmix64
    rng = np.random.default_rng(10327)
    nt = 64
    sizes = np.round(2.0 ** (16 + 8 * rng.random(nt))).astype(np.int64)
    srv = dg.DyCuckooServer(sizes.tolist(), key_bytes=8, value_bytes=4,
                            hbm_cap_bytes=120 << 30)

    def in_class_np(k):
        return (k & np.uint64(63)) == 0

    maps = [O.Map() for _ in range(nt)]
    for i in range(nt):
        kd = splitmix64(torch.arange(int(sizes[i]), device="cuda", dtype=torch.int64), 1)
        vd = torch.randint(0, 1 << 30, (int(sizes[i]),), device="cuda", dtype=torch.int32)
        srv.table(i).insert(kd, vd, unique=True, new_keys=True)
        s = (kd & 63) == 0
        maps[i].insert(_u64(kd[s]), _u32(vd[s]).astype(np.uint64))
    torch.cuda.synchronize()
    zipf = np.arange(1, nt + 1) ** -0.9
    zipf /= zipf.sum()
    reqs = []
    for q in range(3000):
        tn = int(rng.choice(nt, p=zipf))
        n = int(round(2.0 ** (5 + 11 * rng.random())))
        u = rng.random(n)
        ops = np.where(u < 0.7, 0, np.where(u < 0.9, 1, 2)).astype(np.uint8)
        j = np.where(ops == 1, rng.integers(0, 1 << 25, n), rng.integers(0, 1 << 17, n))
        keys = _u64(splitmix64(torch.from_numpy(j.astype(np.int64)).cuda(), 1))
        vals = rng.integers(0, 1 << 30, n).astype(np.uint32)
        reqs.append((q, tn, ops, keys, vals))
    results = {}
    lock = threading.Lock()

    def worker(wk):
        mine = [r for r in reqs if r[1] % 4 == wk]  # a tenant always from one thread
        tickets = [(r[0], srv.submit(r[1], r[2], r[3], r[4])) for r in mine]
        for q, tk in tickets:
            st, out, hits, _ = srv.wait(tk)
            with lock:
                results[q] = (st, out.copy(), hits.copy())

    ths = [threading.Thread(target=worker, args=(wk,)) for wk in range(4)]
    for th in ths:
        th.start()
    for th in ths:
        th.join()
    stats = srv.stats()
    assert stats["steps"] < len(reqs), "requests were not coalesced"
    checked = 0
    for q, tn, ops, keys, vals in reqs:  # submission order within each tenant
        st, out, hits = results[q]
        assert st == 0, (q, st)
        m = in_class_np(keys)
        ov, oh = maps[tn].apply(ops[m], keys[m], vals[m].astype(np.uint64))
        assert np.array_equal(hits[m], oh), "request %d: hit bits differ" % q
        assert np.array_equal(out[m].astype(np.uint64), ov), "request %d: values differ" % q
        checked += int(m.sum())
    for i in range(nt):
        kk, vv = _export_class(srv.table(i), lambda k: (k & 63) == 0, torch)
        _same_contents(kk, vv, maps[i], "tenant %d" % i)
    assert checked > 3e5, checked
    srv.close()
