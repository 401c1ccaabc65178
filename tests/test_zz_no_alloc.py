"""dyc_erase_noalloc: the erase entry point that allocates nothing.

Some callers cannot allocate device memory while they run (an engine whose
own allocator owns all of HBM, or a latency-bound path that cannot take an
allocation's synchronisation). For them dyc_erase_noalloc takes its
batch-dedup scratch from a fixed array in the library. This checks, through
the C ABI, that it returns exactly what dyc_erase returns -- erased bits,
erased count and the table contents afterwards -- on two calls in a row,
that the library makes no device or pinned allocation during those calls
(its own allocation counter, which also sees allocations its memory pool
could serve without the device's free memory moving) and that device free
memory does not move either, and that a batch above the limit is refused
without touching the table.

Kept in its own file so it is collected last.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import assert_same_contents, to_dev, unique_u32, unique_u64

pytestmark = pytest.mark.gpu

LIMIT = 1 << 18


def _mem_free():
    cudart = C.CDLL("libcudart.so.13")
    free, total = C.c_size_t(), C.c_size_t()
    assert cudart.cudaMemGetInfo(C.byref(free), C.byref(total)) == 0
    return free.value


def _allocs(L):
    n = C.c_uint64()
    assert L.dyc_debug_alloc_count(C.byref(n)) == 0
    return n.value


def _erase(L, fn, t, keys_dev, bits_dev, stream):
    cnt = C.c_uint64()
    flags = 4  # DYC_FLAG_NO_RESIZE for the allocating form too, so both do the same work
    rc = getattr(L, fn)(t.handle, C.c_void_p(keys_dev.data_ptr()), keys_dev.numel(),
                        C.c_void_p(bits_dev.data_ptr()), C.byref(cnt), flags, stream)
    assert rc == 0, L.dyc_last_error()
    return int(cnt.value)


@pytest.mark.parametrize("key_bytes", [4, 8])
def test_noalloc_erase_matches_erase_on_two_calls(key_bytes):
    import torch

    import databases_gpu_gb300 as dg
    L = dg.lib()
    n = 200_000
    if key_bytes == 4:
        keys = unique_u32(n, seed=314)
        vals = keys ^ np.uint32(0x13579BDF)
        other = unique_u32(4000, seed=2718)
    else:
        keys = unique_u64(n, seed=314)
        vals = keys ^ np.uint64(0x13579BDF2468ACE0)
        other = unique_u64(4000, seed=2718) ^ np.uint64(1 << 63)
    rng = np.random.default_rng(5)
    # two erase batches with repeats, misses and key 0; the second overlaps the first
    b1 = np.concatenate([rng.choice(keys, 90_000), other[:2000], np.zeros(3, keys.dtype)])
    b2 = np.concatenate([rng.choice(keys, 120_000), other[2000:]])
    rng.shuffle(b1)
    rng.shuffle(b2)

    a = dg.DyCuckoo(n * 2, key_bytes=key_bytes)       # erased with dyc_erase
    b = dg.DyCuckoo(n * 2, key_bytes=key_bytes)       # erased with dyc_erase_noalloc
    m = O.Map()
    for t in (a, b):
        t.insert(to_dev(keys), to_dev(vals))
    m.insert(keys, vals)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    batches = [to_dev(b1), to_dev(b2)]
    bits = [torch.zeros((x.size + 31) // 32, dtype=torch.int32, device="cuda") for x in (b1, b2)
            for _ in range(2)]
    # first call on this device does the one-time set-up; a warm-up with no keys
    # to erase makes every later call a steady-state one
    warm = to_dev(np.array([other[0], other[1]], keys.dtype))
    wbits = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert _erase(L, "dyc_erase_noalloc", b, warm, wbits, stream) == 0
    torch.cuda.synchronize()

    got = []
    new_allocs = []
    free_before = _mem_free()
    for i, kb in enumerate(batches):
        c_ref = _erase(L, "dyc_erase", a, kb, bits[2 * i], stream)
        n0 = _allocs(L)
        c_new = _erase(L, "dyc_erase_noalloc", b, kb, bits[2 * i + 1], stream)
        new_allocs.append(_allocs(L) - n0)
        got.append((c_ref, c_new))
    torch.cuda.synchronize()
    free_after_b = _mem_free()

    for i, (c_ref, c_new) in enumerate(got):
        assert c_new == c_ref, "call %d: erased %d vs %d" % (i, c_new, c_ref)
        assert torch.equal(bits[2 * i], bits[2 * i + 1]), "call %d: erased bits differ" % i
    # and both agree with the oracle's first-occurrence rule
    for i, x in enumerate((b1, b2)):
        _, oh = m.erase(x)
        assert got[i][1] == int(oh.sum())
        assert np.array_equal(dg.unpack_bits(bits[2 * i + 1], x.size), oh)
    assert_same_contents(a, m, "dyc_erase")
    assert_same_contents(b, m, "dyc_erase_noalloc")
    # the no-allocation calls made no allocation of the library's own
    assert new_allocs == [0, 0], new_allocs
    # and nothing in this window allocated device memory at all (dyc_erase
    # reuses scratch sized by its first call): free memory must not move
    assert free_after_b == free_before, (free_before, free_after_b)
    a.close()
    b.close()


def test_noalloc_erase_rejects_oversized_batch():
    import torch

    import databases_gpu_gb300 as dg
    L = dg.lib()
    keys = unique_u32(1000, seed=9)
    t = dg.DyCuckoo(4000)
    t.insert(to_dev(keys), to_dev(keys))
    big = torch.zeros(LIMIT + 1, dtype=torch.int32, device="cuda")
    big[:1000] = to_dev(keys)
    cnt = C.c_uint64(7)
    rc = L.dyc_erase_noalloc(t.handle, C.c_void_p(big.data_ptr()), LIMIT + 1, None,
                             C.byref(cnt), 0, C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 2  # DYC_EINVAL
    assert b"at most 262144" in L.dyc_last_error()
    assert cnt.value == 0
    assert t.size == 1000
    m = O.Map()
    m.insert(keys, keys)
    assert_same_contents(t, m, "after refused call")
    t.close()
