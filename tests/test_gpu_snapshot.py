"""GPU tests of table snapshot / restore (dyc_snapshot, dyc_restore): a
restored table has the same layout, contents and behaviour, a damaged
payload is refused, and snapshots go through files."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import assert_same_contents, find_and_compare, to_dev, unique_u32, unique_u64

pytestmark = pytest.mark.gpu


def _dg():
    import databases_gpu_gb300 as dg
    return dg


@pytest.mark.parametrize("kb,sb", [(4, 128), (4, 32), (8, 128)])
def test_snapshot_round_trip(kb, sb, tmp_path):
    dg = _dg()
    n = 1 << 16
    keys = unique_u32(2 * n, seed=71) if kb == 4 else unique_u64(2 * n, seed=71)
    vals = (np.arange(2 * n) * 7 + 1).astype(keys.dtype) & keys.dtype.type(0x7FFFFFFF)
    t = dg.DyCuckoo(1000, key_bytes=kb, value_bytes=kb, bucket_bytes=sb)
    m = O.Map()
    t.insert(to_dev(keys[:n]), to_dev(vals[:n]))           # grows through upsizes
    t.erase(to_dev(keys[: n // 3]))
    m.insert(keys[:n], vals[:n])
    m.erase(keys[: n // 3])
    buf = t.snapshot()
    r = dg.DyCuckoo.restore(buf)
    assert r.layout() == t.layout() and r.size == t.size and r.capacity == t.capacity
    for i in range(len(t.layout())):
        assert np.array_equal(r.subtable(i, with_meta=True), t.subtable(i, with_meta=True))
    assert_same_contents(r, m, "restored")
    find_and_compare(r, m, keys[: n + n // 2], "finds after restore")
    # the restored table keeps working: inserts, erases, resizes
    r.insert(to_dev(keys[n:]), to_dev(vals[n:]))
    m.insert(keys[n:], vals[n:])
    assert_same_contents(r, m, "restored then grown")
    # through a file
    path = str(tmp_path / "t.dyc")
    r.save(path)
    f = dg.DyCuckoo.load(path)
    assert_same_contents(f, m, "loaded from file")
    for x in (t, r, f):
        x.close()


def test_snapshot_refuses_damaged_payload():
    dg = _dg()
    keys = unique_u32(5000, seed=3)
    t = dg.DyCuckoo(5000)
    t.insert(to_dev(keys), to_dev(keys))
    buf = t.snapshot()
    bad = buf.copy()
    bad[256 + 1000] ^= 0x40
    with pytest.raises(dg.DycError) as e:
        dg.DyCuckoo.restore(bad)
    assert "checksum" in str(e.value)
    ok = dg.DyCuckoo.restore(buf)
    assert ok.size == 5000
    t.close()
    ok.close()
