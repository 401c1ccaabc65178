"""GPU parity of wide-value tables (dyc_wide_*) against the oracle.

Every value is a deterministic expansion of a 64-bit id (value_bytes of
splitmix64 words), and the oracle map stores the ids: the GPU's returned
bytes must equal the expansion of the id the oracle holds (zeros on a miss).
Covers repeated keys in a batch (last insert wins, first erase removes),
erase returning values, handle reuse after erases, growth of the value heap
and of the table, downsizes, u32 and u64 keys, and several value widths.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import to_dev, to_host, unique_u32, unique_u64

pytestmark = pytest.mark.gpu


def _dg():
    import databases_gpu_gb300 as dg
    return dg


def expand(ids: np.ndarray, vbytes: int) -> np.ndarray:
    """(n, vbytes/4) uint32 rows: splitmix64(id * 4099 + word) words; id 0 -> zeros."""
    words = vbytes // 4
    w = np.arange((words + 1) // 2, dtype=np.uint64)
    with np.errstate(over="ignore"):
        x = ids[:, None].astype(np.uint64) * np.uint64(4099) + w[None, :] + \
            np.uint64(0x9E3779B97F4A7C15)
        x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        x = x ^ (x >> np.uint64(31))
    rows = np.ascontiguousarray(x).view(np.uint32).reshape(ids.size, -1)[:, :words].copy()
    rows[ids == 0] = 0
    return rows


def _rows_dev(rows):
    import torch
    return torch.from_numpy(np.ascontiguousarray(rows).view(np.int32)).cuda()


def _check_find(w, m, q, vbytes, label):
    out, bits = w.find(to_dev(q))
    got = out.cpu().numpy().view(np.uint32)
    hits = _dg().unpack_bits(bits, q.size)
    ov, oh = m.find(q.astype(np.uint64))
    assert np.array_equal(hits, oh), "%s: hit bits differ" % label
    assert np.array_equal(got, expand(ov, vbytes)), "%s: values differ" % label


@pytest.mark.parametrize("kb,vbytes", [(4, 4), (4, 40), (4, 128), (8, 16), (8, 256)])
def test_wide_matches_oracle(kb, vbytes):
    rng = np.random.default_rng(vbytes + kb)
    pool = unique_u32(40000, seed=5) if kb == 4 else unique_u64(40000, seed=5)
    w = _dg().DyCuckooWide(1000, vbytes, key_bytes=kb, min_downsize_capacity=0)
    m = O.Map()
    next_id = 1
    for b in range(6):
        n = 30000
        keys = pool[rng.integers(0, pool.size, n)]       # repeats inside the batch
        ids = np.arange(next_id, next_id + n, dtype=np.uint64)
        next_id += n
        st = w.insert(to_dev(keys), _rows_dev(expand(ids, vbytes)))
        m.insert(keys, ids)
        assert st["inserted"] + st["updated"] == np.unique(keys).size
        _check_find(w, m, pool[rng.integers(0, pool.size, 20000)], vbytes, "batch %d find" % b)
        # erase some keys, with repeats: the removed values come back
        er = pool[rng.integers(0, pool.size, 8000)]
        ov, oh = m.erase(er.astype(np.uint64))
        cnt, out, bits = w.erase(to_dev(er))
        assert cnt == int(oh.sum())
        assert np.array_equal(_dg().unpack_bits(bits, er.size), oh)
        assert np.array_equal(out.cpu().numpy().view(np.uint32), expand(ov, vbytes))
        assert w.size == len(m)
    # full contents
    k, v = w.export()
    ok_, ov_ = m.export()
    assert np.array_equal(to_host(k, kb).astype(np.uint64), ok_)
    assert np.array_equal(v.cpu().numpy().view(np.uint32), expand(ov_, vbytes))
    w.close()
