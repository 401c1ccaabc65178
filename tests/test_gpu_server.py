"""GPU tests of the request server (dyc_server_*): continuous batching gives
every request exactly the results it gets alone.

Requests for u64-key / u32-value tenants are submitted concurrently from
several threads (each tenant always from the same thread, so its submission
order is fixed), coalesced into shared device steps by the server, and
compared with (a) the same requests run one at a time, (b) the per-request
path without coalescing and (c) the oracle applying each tenant's requests in
order. Admission under a small HBM cap rejects a request that can never fit
and still serves the others.
"""
import threading
import time

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _dg():
    import databases_gpu_gb300 as dg
    return dg


def _requests(seed, ntenants, count, max_log2=12):
    rng = np.random.default_rng(seed)
    pools = [rng.integers(1, 1 << 62, 3000, dtype=np.int64).astype(np.uint64)
             for _ in range(ntenants)]
    reqs = []
    for i in range(count):
        t = int(rng.integers(0, ntenants))
        n = int(round(2 ** rng.uniform(5, max_log2)))
        ops = rng.choice(np.array([0, 1, 2], np.uint8), size=n, p=[0.7, 0.2, 0.1])
        keys = pools[t][rng.integers(0, pools[t].size, n)]
        keys[rng.random(n) < 0.01] = 0  # some key-0 ops
        vals = rng.integers(0, 1 << 32, n, dtype=np.int64).astype(np.uint32)
        reqs.append((i, t, ops, keys, vals))
    return reqs


def _run_mixed(srv, reqs, nthreads=4):
    res = {}
    lock = threading.Lock()

    def worker(w):
        rng = np.random.default_rng(100 + w)
        mine = [r for r in reqs if r[1] % nthreads == w]
        tickets = []
        for (i, t, ops, keys, vals) in mine:
            tickets.append((i, srv.submit(t, ops, keys, vals)))
            if rng.random() < 0.3:
                time.sleep(rng.uniform(0, 0.002))
        for i, tk in tickets:
            st, out, bits, lat = srv.wait(tk)
            with lock:
                res[i] = (st, out.copy(), bits.copy())

    ths = [threading.Thread(target=worker, args=(w,)) for w in range(nthreads)]
    for th in ths:
        th.start()
    for th in ths:
        th.join()
    return res


def _run_alone(srv, reqs):
    res = {}
    for (i, t, ops, keys, vals) in reqs:
        st, out, bits, lat = srv.wait(srv.submit(t, ops, keys, vals))
        res[i] = (st, out.copy(), bits.copy())
    return res


def test_server_results_same_alone_and_in_the_mix():
    nt = 12
    sizes = [1 << (8 + t % 6) for t in range(nt)]
    reqs = _requests(1, nt, 300)
    mixed = _dg().DyCuckooServer(sizes, max_step_ops=1 << 15)
    r_mix = _run_mixed(mixed, reqs)
    st = mixed.stats()
    assert st["requests"] == len(reqs) and st["rejected"] == 0
    assert st["steps"] < len(reqs), "requests were never coalesced into shared steps"
    alone = _dg().DyCuckooServer(sizes, max_step_ops=1 << 15)
    r_alone = _run_alone(alone, reqs)
    plain = _dg().DyCuckooServer(sizes, max_step_ops=1 << 15, coalesce=False)
    r_plain = _run_mixed(plain, reqs)
    # the oracle: each tenant's requests in submission order (request order
    # within a tenant is the same in every run)
    maps = [O.Map() for _ in range(nt)]
    for (i, t, ops, keys, vals) in reqs:
        ov, oh = maps[t].apply(ops, keys, vals.astype(np.uint64))
        for name, r in (("mixed", r_mix), ("alone", r_alone), ("per-request", r_plain)):
            s, out, bits = r[i]
            assert s == 0, "%s request %d status %d" % (name, i, s)
            assert np.array_equal(bits, oh), "%s request %d: hit bits differ" % (name, i)
            assert np.array_equal(out.astype(np.uint64), ov & np.uint64(0xFFFFFFFF)), \
                "%s request %d: values differ" % (name, i)
    for srv in (mixed, alone, plain):
        srv.close()


def test_server_admission_rejects_what_can_never_fit():
    srv = _dg().DyCuckooServer([1024] * 4, max_step_ops=1 << 13)
    # after one step: the set's first round allocates every member's upsize
    # target (spare), which counts against the cap from then on
    st, _, _, _ = srv.wait(srv.submit(0, np.zeros(1, np.uint8), np.ones(1, np.uint64),
                                      np.zeros(1, np.uint32)))
    assert st == 0
    base = srv.stats()["device_bytes"]
    srv.close()
    # room for the growth of about 1000 inserts (40 bytes each with headroom)
    srv = _dg().DyCuckooServer([1024] * 4, max_step_ops=1 << 13, hbm_cap_bytes=base + 40_000)
    rng = np.random.default_rng(3)
    big_keys = rng.integers(1, 1 << 62, 5000, dtype=np.int64).astype(np.uint64)
    big = srv.submit(0, np.ones(5000, np.uint8), big_keys, np.ones(5000, np.uint32))
    st, _, _, _ = srv.wait(big)
    assert st == 1  # DYC_ENOMEM: 5000 inserts can never fit under the cap
    small = []
    for t in range(4):
        k = rng.integers(1, 1 << 62, 200, dtype=np.int64).astype(np.uint64)
        small.append((t, k, srv.submit(t, np.ones(200, np.uint8), k, np.arange(200, dtype=np.uint32))))
    for t, k, tk in small:
        st, out, bits, _ = srv.wait(tk)
        assert st == 0 and not bits.any()
    for t, k, _ in small:
        tk = srv.submit(t, np.zeros(200, np.uint8), k, np.zeros(200, np.uint32))
        st, out, bits, _ = srv.wait(tk)
        assert st == 0 and bits.all() and np.array_equal(out, np.arange(200, dtype=np.uint32))
    s = srv.stats()
    assert s["rejected"] == 1
    srv.close()
