"""Pin the oracle to outputs of the reference's own code.

tests/golden/reference_kat.npz was produced by tests/golden/make_golden.py,
which compiles the reference's hash functions, pair maps, makeEntry, sizing,
resize target choice, MT19937 and key generators (GPU/dyhash/cuckoo.cu,
api.cpp, diff_hash_num_pos_fun.cpp, mt19937ar.cpp, random_numbers.cpp) and
records what they return.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O

KAT = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_kat.npz"))
L = O.lib()


def test_mt19937_streams():
    for seed in (10327, 5489):
        ref = KAT["mt_%d" % seed]
        mt = O.MT19937(seed)
        assert np.array_equal(mt.fill_u32(ref.size), ref)


@pytest.mark.parametrize("i", [1, 2, 3, 4, 5])
def test_hash_functions(i):
    keys = KAT["hash_keys"]
    f = getattr(L, "orc_hash%d" % i)
    got = np.array([f(int(k)) for k in keys], np.uint32)
    assert np.array_equal(got, KAT["hash%d" % i])


def test_hash_function_mod_chain():
    keys = KAT["hash_keys"]
    for t in range(4):
        for j, nb in enumerate(KAT["hf_nbuckets"]):
            got = np.array([L.orc_bucket_of(int(k), t, int(nb)) for k in keys], np.uint32)
            assert np.array_equal(got, KAT["hash_function"][t, j]), (t, nb)


def test_pair_choice_four_subtables():
    keys = KAT["hash_keys"]
    got = np.array([L.orc_choose_hash(int(k), 4) for k in keys], np.uint32)
    assert np.array_equal(got, KAT["choose4"])
    assert np.array_equal([L.orc_pos1(p, 4) for p in range(6)], KAT["pos1_4"])
    assert np.array_equal([L.orc_pos2(p, 4) for p in range(6)], KAT["pos2_4"])
    # get_pos: the other table of the pair, or pos1 when `pre` is not pos1
    for p in range(6):
        for j, pre in enumerate((0, 1, 2, 3, 100)):
            exp = L.orc_pos2(p, 4) if pre == L.orc_pos1(p, 4) else L.orc_pos1(p, 4)
            assert exp == KAT["get_pos4"][p, j]


@pytest.mark.parametrize("d,npairs", [(2, 2), (3, 3), (5, 10)])
def test_pair_choice_variants(d, npairs):
    keys = KAT["hash_keys"]
    got = np.array([L.orc_choose_hash(int(k), d) for k in keys], np.uint32)
    assert np.array_equal(got, KAT["choose_d%d" % d])
    assert np.array_equal([L.orc_pos1(p, d) for p in range(npairs)], KAT["pos1_d%d" % d])
    assert np.array_equal([L.orc_pos2(p, d) for p in range(npairs)], KAT["pos2_d%d" % d])


def test_pair_maps_cover_all_pairs():
    # d = 6 comes from a snippet that does not compile (GPU/dyhash/
    # diff_hash_num_pos_fun.cpp:152-188 uses `case 0,1,...:` labels), so it is
    # pinned structurally: every unordered pair of subtables exactly once.
    for d, npairs in ((2, 2), (3, 3), (4, 6), (5, 10), (6, 15)):
        pairs = {tuple(sorted((L.orc_pos1(p, d), L.orc_pos2(p, d)))) for p in range(npairs)}
        assert all(a != b and 0 <= a < d and 0 <= b < d for a, b in pairs)
        if d > 2:
            assert len(pairs) == d * (d - 1) // 2


def test_make_entry_sign_extension():
    # the oracle's reference mode packs like cuckoo.cu:337-345
    for k, v, e in zip(KAT["entry_k"], KAT["entry_v"], KAT["entry"]):
        exp = ((int(k) << 32) + (int(v) - (1 << 32) if v >= (1 << 31) else int(v))) % (1 << 64)
        assert exp == int(e)


def test_sizing():
    for x, p in enumerate(KAT["is_prime"]):
        assert L.orc_is_prime(x) == p, x
    for n, p in zip(KAT["next_prime_in"], KAT["next_prime"]):
        assert L.orc_next_prime(int(n)) == p
    for s, b in zip(KAT["size_in"], KAT["subtable_buckets"]):
        s = int(s) & 0xFFFFFFFF  # hashAPI takes a 32-bit size
        assert L.orc_subtable_buckets(s, 4, 16) == b, s


def test_resize_target_choice():
    for lay, up, down in zip(KAT["layouts"], KAT["pick_up"], KAT["pick_down"]):
        nb = np.ascontiguousarray(lay, np.uint32)
        assert L.orc_pick_up_nb(nb, 4) == up, lay
        assert L.orc_pick_down_nb(nb, 4) == down, lay


def test_resize_choice_sequence_on_oracle_table():
    # up from equal sizes walks 0,1,2,3 then 0 again; down mirrors it
    t = O.RefCuckoo(64 * 40, 4, 16)
    seen = [t.resize_up() for _ in range(5)] + [t.resize_down() for _ in range(6)]
    assert seen == [0, 1, 2, 3, 0, 0, 3, 2, 1, 0, 3]


def test_unique_generator():
    for n in (100, 1024, 20000):
        ref = KAT["unique_10327_%d" % n]
        got = O.MT19937(10327).unique_ref(2 * n)
        assert np.array_equal(got, ref)
        assert np.unique(ref).size == ref.size


def test_query_generator():
    n = 5000
    mt = O.MT19937(4242)
    pool = mt.unique_ref(2 * n)
    assert np.array_equal(pool, KAT["queries_pool_before"])
    q = mt.queries(n, 0.5, pool)
    assert np.array_equal(q, KAT["queries_05"])
    assert np.array_equal(pool, KAT["queries_pool_after"])
