"""Differential parity against the reference's own GPU kernels.

The reference's cuckoo_insert / cuckoo_search / cuckoo_delete and its resize
kernels (GPU/dyhash/cuckoo.cu:324-788, compiled for sm_103a by
oracle/build_ref.py, run through oracle/ref_gpu.py with the reference's grid)
are run on the same seeded inputs as the library (through its C ABI) and the
oracle. Inputs stay in the domain where the reference is well defined:
unique nonzero keys, values below 2^31 (its makeEntry sign-extends larger
ones), no update of existing keys.

The reference drops the entry left at the end of a 15-step eviction chain
(cuckoo.cu:422-431) and a downsize residual it cannot place (:714-722), and
which entry is dropped depends on the order its warps run in. So:

* where the reference dropped nothing (its rehash flag is 0), its contents
  and every search result equal the library's and the oracle's bit for bit;
* where it dropped entries, everything it kept equals the library's value
  for that key, its search answers exactly from what it kept, and the keys
  it lost are the only difference (their count is the reference's loss).

Every entry the reference kernels placed sits in one of the two buckets the
oracle's restatement of its hash functions and pair map names for the key,
which pins that restatement to the reference's compiled kernels as well.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import assert_same_contents, to_dev, unique_u32

pytestmark = pytest.mark.gpu


def _ref_gpu():
    from oracle import ref_gpu
    if not ref_gpu.available():
        pytest.skip("reference GPU kernels not staged (oracle/build_ref.py)")
    return ref_gpu


def _ref_map(ref):
    """The reference table's contents as a dict-free sorted pair of arrays;
    fails if a key sits in two slots (unique inputs never do that)."""
    k, v = ref.export()
    order = np.argsort(k, kind="stable")
    k, v = k[order], v[order]
    assert np.all(k[1:] != k[:-1]), "reference table holds a key twice"
    return k, v


def _lookup(sk, sv, q):
    """Value of each q in the sorted (sk, sv) map, and a found mask."""
    if sk.size == 0:
        return np.zeros(q.size, np.uint32), np.zeros(q.size, bool)
    pos = np.minimum(np.searchsorted(sk, q), sk.size - 1)
    found = sk[pos] == q
    return np.where(found, sv[pos], 0).astype(np.uint32), found


def _check_placement(ref):
    """Every occupied slot of the reference table is one of its key's two
    candidate buckets under the oracle's hashes (cuckoo.cu:76-90, :190-213)."""
    nb = ref.layout()
    for t, sub in enumerate(ref.subtables):
        a = sub.cpu().numpy().view(np.uint64).reshape(nb[t], ref.SLOTS)
        b_idx, _ = np.nonzero(a)
        keys = (a[a != 0] >> np.uint64(32)).astype(np.uint32)
        t1, b1, t2, b2 = O.hash_batch(keys, 4, nb)
        ok = ((t1 == t) & (b1 == b_idx)) | ((t2 == t) & (b2 == b_idx))
        assert ok.all(), "subtable %d: %d entries outside their candidate buckets" % (
            t, int((~ok).sum()))


def _compare(ref, ours, omap, queries, label, exact):
    """Reference contents and search vs the library (find) and the oracle."""
    from databases_gpu_gb300 import unpack_bits
    rk, rv = _ref_map(ref)
    ok_, ov_ = omap.export()
    ok32, ov32 = ok_.astype(np.uint32), ov_.astype(np.uint32)
    # everything the reference kept is in the oracle with the same value
    val, found = _lookup(ok32, ov32, rk)
    assert found.all(), "%s: reference holds %d keys the oracle does not" % (label, int((~found).sum()))
    assert np.array_equal(val, rv), "%s: %d reference values differ from the oracle" % (
        label, int((val != rv).sum()))
    lost = ok32.size - rk.size
    if exact:
        assert lost == 0, "%s: reference lost %d entries" % (label, lost)
    # reference search answers from what it holds
    qd = to_dev(queries)
    r_out = ref.search(qd).cpu().numpy().view(np.uint32)
    exp_r, in_ref = _lookup(rk, rv, queries)
    assert np.array_equal(r_out, exp_r), "%s: reference search differs from its own contents" % label
    # the library agrees with the reference on every key the reference kept,
    # and with the oracle everywhere
    g_out, g_bits = ours.find(qd)
    g_val = g_out.cpu().numpy().view(np.uint32)
    g_hit = unpack_bits(g_bits, queries.size)
    assert np.array_equal(g_hit[in_ref], np.ones(int(in_ref.sum()), bool)), label
    assert np.array_equal(g_val[in_ref], r_out[in_ref]), "%s: values differ from the reference" % label
    o_val, o_hit = omap.find(queries.astype(np.uint64))
    assert np.array_equal(g_hit, o_hit) and np.array_equal(g_val, o_val.astype(np.uint32)), label
    # outside the reference's losses, hit or miss agree too
    only_ours = g_hit & ~in_ref
    assert int(only_ours.sum()) <= lost, label
    if exact:
        assert np.array_equal(g_hit, in_ref) and np.array_equal(g_val, r_out), label
    return lost


@pytest.mark.parametrize("log2n,lf", [(16, 0.85), (20, 0.85), (18, 0.6)])
def test_reference_kernels_insert_search_delete(log2n, lf):
    """The measurement plan's plain sequence: n unique keys inserted in one
    batch into hashAPI(n / lf), finds with 50 % hits, delete n/2, re-find.
    Load factor 0.85 (its first case) loses a few entries in the reference;
    at 0.6 it loses none and everything must match exactly."""
    import databases_gpu_gb300 as dg
    ref_gpu = _ref_gpu()
    n = 1 << log2n
    pool = unique_u32(2 * n)
    keys = pool[:n]
    vals = (np.arange(n, dtype=np.uint32) * 3 + 4) & np.uint32(0x7FFFFFFF)
    size = int(n / lf)
    ref = ref_gpu.RefGpuTable(size)
    ours = dg.DyCuckoo(size)
    omap = O.Map(n)
    flag = ref.insert(to_dev(keys), to_dev(vals))
    ours.insert(to_dev(keys), to_dev(vals))
    omap.insert(keys, vals)
    assert_same_contents(ours, omap, "library after insert")
    _check_placement(ref)
    queries = pool.copy()
    O.MT19937(7).shuffle(queries)
    lost = _compare(ref, ours, omap, queries, "after insert", exact=(lf <= 0.6))
    assert (flag != 0) == (lost > 0), (flag, lost)
    # delete half of the inserted keys in all three
    dk = keys[: n // 2]
    ref.delete(to_dev(dk))
    erased = ours.erase(to_dev(dk))
    _, eh = omap.erase(dk)
    assert erased == int(eh.sum()) == n // 2
    assert_same_contents(ours, omap, "library after delete")
    lost_after = _compare(ref, ours, omap, queries, "after delete", exact=(lf <= 0.6))
    # deleting never brings a lost key back and never loses another
    assert lost_after <= lost
    ours.close()


def test_reference_kernels_resize_round_trip():
    """Upsizes and downsizes of the subtable hashAPI::resize_up / resize_low
    pick (api.cpp:112-173), run by the reference's resize kernels and by the
    library on tables holding the same keys: an upsize moves every entry
    (the reference loses none), and after each downsize the library still
    matches the oracle exactly while the reference matches on all it kept."""
    import databases_gpu_gb300 as dg
    ref_gpu = _ref_gpu()
    n = 1 << 16
    pool = unique_u32(2 * n, seed=4242)
    keys = pool[:n]
    vals = np.arange(1, n + 1, dtype=np.uint32)
    size = int(n / 0.6)
    ref = ref_gpu.RefGpuTable(size)
    ours = dg.DyCuckoo(size, auto_resize=False)
    omap = O.Map(n)
    assert ref.insert(to_dev(keys), to_dev(vals)) == 0
    ours.insert(to_dev(keys), to_dev(vals))
    omap.insert(keys, vals)
    for step in range(3):
        ref.resize_up(ref.pick_up())
        ours.resize_up()
        _check_placement(ref)
        assert_same_contents(ours, omap, "library upsize %d" % step)
        _compare(ref, ours, omap, pool, "upsize %d" % step, exact=True)
    downs = 0
    while downs < 3:
        t = ref.pick_down()
        if ref.layout()[t] % 2:
            break  # the reference's downsize needs an even bucket count
        ref.resize_down(t)
        ours.resize_down()
        downs += 1
        _check_placement(ref)
        assert_same_contents(ours, omap, "library downsize %d" % downs)
        _compare(ref, ours, omap, pool, "downsize %d" % downs, exact=False)
    assert downs >= 1
    ours.close()
