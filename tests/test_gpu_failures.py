"""Failure paths that must not lose entries, driven by host-side injection.

dyc_debug_inject makes the n-th allocation from the library pool fail as if
the device were out of memory, or makes the downsize kernel's bounded
tile-copy waits give up at once. Nothing here faults, traps or hangs the
GPU: the allocation failure is returned by the host code before any kernel
sees it, and a wait that gives up returns a status the host reads (the
block still waits, with its full bound, for its own copies before it exits).

The reference drops an entry left at the end of an eviction chain
(GPU/dyhash/cuckoo.cu:422-431) and downsize residuals it cannot place
(:714-722). Here such entries are held by the table and placed by the next
call; every check ends with the full contents equal to the oracle's.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import assert_same_contents, find_and_compare, to_dev, unique_u32

pytestmark = pytest.mark.gpu


def _dg():
    import databases_gpu_gb300 as dg
    return dg


@pytest.fixture(autouse=True)
def _clear_injection():
    from databases_gpu_gb300 import _lib
    _lib.lib().dyc_debug_inject(_lib.INJECT_RESET, 0)
    yield
    _lib.lib().dyc_debug_inject(_lib.INJECT_RESET, 0)


def _inject(kind, n):
    from databases_gpu_gb300 import _lib
    assert _lib.lib().dyc_debug_inject(kind, n) == 0


def _raises(status, fn):
    dg = _dg()
    with pytest.raises(dg.DycError) as ei:
        fn()
    assert ei.value.status == status, ei.value
    return ei.value


def test_insert_whose_upsize_fails_holds_entries_until_the_next_call():
    """An insert that overflows its eviction chains needs an upsize; the
    first pool allocation fails: DYC_ENOMEM, nothing dropped, the unplaced
    entries are held (counted by size, reported in stats) and the next call
    (a find) places them before it runs."""
    from databases_gpu_gb300 import _lib
    dg = _dg()
    n = 1 << 15
    keys = unique_u32(n, seed=71)
    vals = np.arange(1, n + 1, dtype=np.uint32)
    t = dg.DyCuckoo(n, max_evictions=1, auto_resize=False)
    m = O.Map(n)
    m.insert(keys, vals)
    _inject(_lib.INJECT_POOL_ALLOC, 1)
    err = _raises(_lib.DYC_ENOMEM, lambda: t.insert(to_dev(keys), to_dev(vals)))
    assert "held" in str(err)
    held = t.stats()["held"]
    assert held > 0
    assert t.size == n  # held entries are keys of the table
    # the next call places them (the injection is spent), then finds
    find_and_compare(t, m, keys, "after the held entries were placed")
    assert t.stats()["held"] == 0
    assert_same_contents(t, m, "contents")
    t.close()


@pytest.mark.parametrize("which", [1, 2, 3])
def test_downsize_allocation_failure_leaves_the_table_unchanged(which):
    """The downsize allocates its new subtable and two entry lists; any of
    the three failing returns DYC_ENOMEM with the table exactly as before
    (layout, size, contents), and a downsize afterwards works."""
    from databases_gpu_gb300 import _lib
    dg = _dg()
    n = 1 << 15
    keys = unique_u32(n, seed=72)
    vals = np.arange(1, n + 1, dtype=np.uint32)
    t = dg.DyCuckoo(4 * n, auto_resize=False)
    m = O.Map(n)
    t.insert(to_dev(keys), to_dev(vals))
    m.insert(keys, vals)
    layout = t.layout()
    _inject(_lib.INJECT_POOL_ALLOC, which)
    _raises(_lib.DYC_ENOMEM, t.resize_down)
    assert t.layout() == layout and t.size == n
    assert_same_contents(t, m, "after the failed downsize")
    t.resize_down()
    assert sum(t.layout()) < sum(layout)
    assert_same_contents(t, m, "after the downsize")
    t.close()


def test_downsize_whose_placement_upsize_fails_holds_entries():
    """A downsize of a full table leaves entries its eviction walks cannot
    place without an upsize; that upsize (the fourth pool allocation of the
    call, after the new subtable and two lists) fails: DYC_ENOMEM, the
    entries are held and counted, and the next call places them. Downsizes
    are repeated until one needs the upsize."""
    from databases_gpu_gb300 import _lib
    dg = _dg()
    n = 1 << 15
    keys = unique_u32(n, seed=73)
    vals = np.arange(1, n + 1, dtype=np.uint32)
    t = dg.DyCuckoo(n, max_evictions=1, auto_resize=False, upper_load=0.99)
    m = O.Map(n)
    t.insert(to_dev(keys), to_dev(vals))
    m.insert(keys, vals)
    hit = False
    for _ in range(8):
        _inject(_lib.INJECT_RESET, 0)
        _inject(_lib.INJECT_POOL_ALLOC, 4)
        try:
            t.resize_down()
        except dg.DycError as e:
            assert e.status == _lib.DYC_ENOMEM, e
            hit = True
            break
        assert_same_contents(t, m, "after a downsize that needed no upsize")
    assert hit, "no downsize needed an upsize"
    _inject(_lib.INJECT_RESET, 0)
    assert t.stats()["held"] > 0
    assert t.size == n
    find_and_compare(t, m, keys, "after the held entries were placed")
    assert t.stats()["held"] == 0
    assert_same_contents(t, m, "contents")
    t.close()


def test_downsize_wait_timeout_leaves_the_table_unchanged():
    """The merge kernel's tile-copy waits give up at the first poll: the call
    returns DYC_ETIMEOUT, the descriptor still points at the old subtable
    (only read by the kernel) and the contents are intact; with the bound
    restored the downsize works."""
    from databases_gpu_gb300 import _lib
    dg = _dg()
    n = 1 << 15
    keys = unique_u32(n, seed=74)
    vals = np.arange(1, n + 1, dtype=np.uint32)
    t = dg.DyCuckoo(4 * n, auto_resize=False)
    m = O.Map(n)
    t.insert(to_dev(keys), to_dev(vals))
    m.insert(keys, vals)
    layout = t.layout()
    assert all(nb % 2 == 0 for nb in layout)  # the merge kernel (not the odd rehash) runs
    _inject(_lib.INJECT_WAIT_TRIES, 0)
    _raises(_lib.DYC_ETIMEOUT, t.resize_down)
    assert t.layout() == layout and t.size == n
    assert_same_contents(t, m, "after the timed-out downsize")
    find_and_compare(t, m, keys, "finds after the timed-out downsize")
    _inject(_lib.INJECT_RESET, 0)
    t.resize_down()
    assert sum(t.layout()) < sum(layout)
    assert_same_contents(t, m, "after the downsize")
    t.close()


def test_set_places_a_members_held_entries_before_its_batch():
    """A member table of a set holds entries after a failed single-table
    insert; the next set batch places them first, and every op of the batch
    and every table's contents match the oracle."""
    from databases_gpu_gb300 import _lib
    from databases_gpu_gb300.workloads import MultiTableWorkload
    from tests.helpers import to_host
    dg = _dg()
    w = MultiTableWorkload(8, log2_size=(10, 12), log2_batch=(6, 10), seed=75)
    S = dg.DyCuckooSet(w.sizes.numpy(), max_evictions=1)
    maps = [O.Map() for _ in range(S.ntables)]
    for t in range(S.ntables):
        k, v = w.preload(t)
        S.table(t).insert(k, v)
        maps[t].insert(to_host(k, 4), to_host(v, 4))
    # member 0 takes a batch that overflows its chains; its upsize fails
    extra = unique_u32(1 << 13, seed=76)
    extra = extra[~np.isin(extra, maps[0].export()[0].astype(np.uint32))]
    ev = np.arange(7, 7 + extra.size, dtype=np.uint32)
    _inject(_lib.INJECT_POOL_ALLOC, 1)
    _raises(_lib.DYC_ENOMEM, lambda: S.table(0).insert(to_dev(extra), to_dev(ev),
                                                        no_resize=True))
    _inject(_lib.INJECT_RESET, 0)
    maps[0].insert(extra, ev)
    assert S.table(0).stats()["held"] > 0
    ops, keys, vals = w.round()
    out, bits = S.apply(w.offsets, ops, keys, vals, h_offsets=w.offsets_host)
    gv = to_host(out, 4).astype(np.uint64)
    gh = dg.unpack_bits(bits, keys.numel())
    o, k, v = ops.cpu().numpy(), to_host(keys, 4).astype(np.uint64), to_host(vals, 4).astype(np.uint64)
    for t in range(S.ntables):
        a, b = int(w.offsets_host[t]), int(w.offsets_host[t + 1])
        ov, oh = maps[t].apply(o[a:b], k[a:b], v[a:b])
        assert np.array_equal(gh[a:b], oh) and np.array_equal(gv[a:b], ov), "table %d" % t
    for t in range(S.ntables):
        assert_same_contents(S.table(t), maps[t], "table %d" % t)
    assert S.table(0).stats()["held"] == 0
    S.close()


def test_set_member_without_a_spare_is_upsized_by_the_host():
    """A table set applies its upsize policy on the device, from one upsize
    target allocated ahead per member. When that allocation fails (injected:
    the first pool allocation of the round), the member has no spare; the
    device hands the policy to the host for that round, which upsizes it
    before phase B. Every round's results, sizes and capacities equal those
    of a twin set whose host applies the policy, and the oracle's."""
    import torch
    from databases_gpu_gb300 import _lib
    from tests.helpers import to_host
    dg = _dg()
    rng = np.random.default_rng(77)
    nt = 16
    A = dg.DyCuckooSet([2000] * nt, device_upsize=0)
    B = dg.DyCuckooSet([2000] * nt, device_upsize=1)
    _, caps = A.sizes()
    maps = [O.Map() for _ in range(nt)]
    for t in range(nt):
        k = unique_u32(int(0.78 * int(caps[t])), seed=100 + t)
        v = rng.integers(0, 1 << 31, k.size).astype(np.uint32)
        A.table(t).insert(to_dev(k), to_dev(v))
        B.table(t).insert(to_dev(k), to_dev(v))
        maps[t].insert(k, v)
    splits = []
    for r in range(2):
        caps_now = A.sizes()[1].astype(np.int64)
        cnt = (0.16 * caps_now).astype(np.int64)  # new keys: one upsize per member
        off = np.zeros(nt + 1, np.uint32)
        off[1:] = np.cumsum(cnt)
        n = int(off[-1])
        keys = rng.integers((1 << 31) + 1, (1 << 32) - 1, n, dtype=np.uint64).astype(np.uint32)
        ops = np.ones(n, np.uint8)
        vals = rng.integers(0, 1 << 31, n).astype(np.uint32)
        d = lambda a: torch.from_numpy(a.view(np.int32) if a.dtype == np.uint32 else a).cuda()
        if r == 1:
            _inject(_lib.INJECT_POOL_ALLOC, 1)
        oa, ba = A.apply(d(off), d(ops), d(keys), d(vals), h_offsets=off)
        _inject(_lib.INJECT_RESET, 0)
        splits.append(A.stats()["split_phases"])
        ob, bb = B.apply(d(off), d(ops), d(keys), d(vals), h_offsets=off)
        assert bool((oa == ob).all()) and bool((ba == bb).all()), "round %d" % r
        gv = to_host(oa, 4).astype(np.uint64)
        gh = dg.unpack_bits(ba, n)
        for t in range(nt):
            a, b = int(off[t]), int(off[t + 1])
            ov, oh = maps[t].apply(ops[a:b], keys[a:b].astype(np.uint64),
                                   vals[a:b].astype(np.uint64))
            assert np.array_equal(gh[a:b], oh) and np.array_equal(gv[a:b], ov), \
                "round %d table %d" % (r, t)
        sza, capa = A.sizes()
        szb, capb = B.sizes()
        assert np.array_equal(sza, szb) and np.array_equal(capa, capb), "round %d" % r
    # first batch: every member upsized on the device; second: one member had no spare
    assert splits == [0, 1], splits
    for t in range(nt):
        assert_same_contents(A.table(t), maps[t], "table %d" % t)
    A.close()
    B.close()
