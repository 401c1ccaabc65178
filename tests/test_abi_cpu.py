"""CPU-only checks of the C ABI: the library builds, loads, exports every
symbol include/dycuckoo.h declares, and its structs match the header."""
import ctypes as C
import os
import re
import subprocess

import pytest

import databases_gpu_gb300 as dg
from databases_gpu_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "dycuckoo.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(dyc_[a-z_0-9]+)\s*\(", src)))


def test_header_declares_the_exported_surface():
    decl = declared_functions()
    assert decl == sorted(_lib.EXPORTS)


def test_library_exports_every_declared_symbol():
    L = dg.lib()
    for name in declared_functions():
        assert hasattr(L, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", dg.library_path()],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r" T (dyc_\w+)", out))
    assert set(declared_functions()) <= exported


def test_struct_layout_matches_header(tmp_path):
    """Every struct the Python mirror declares has the header's size and field
    offsets (gcc on the header against ctypes)."""
    mirrors = [("dyc_config", _lib.DycConfig), ("dyc_op_stats", _lib.DycOpStats),
               ("dyc_server_config", _lib.DycServerConfig),
               ("dyc_server_stats", _lib.DycServerStats)]
    lines, want = [], []
    for cname, M in mirrors:
        lines.append('printf("%%zu\\n", sizeof(%s));' % cname)
        want.append(C.sizeof(M))
        for f, _ in M._fields_:
            lines.append('printf("%%zu\\n", offsetof(%s, %s));' % (cname, f))
            want.append(getattr(M, f).offset)
    prog = tmp_path / "layout.c"
    prog.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "dycuckoo.h"\n'
                    "int main(void){" + "".join(lines) + "return 0;}\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(prog), "-o", str(exe)],
                   check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    assert got == want


def test_server_config_defaults():
    L = _lib.lib()
    c = _lib.DycServerConfig()
    L.dyc_server_config_default(C.byref(c))
    assert c.hbm_cap_bytes == 0 and c.max_step_ops == 1 << 22 and c.coalesce == 1
    assert c.pool_reserve_bytes == (1 << 64) - 1  # DYC_POOL_RESERVE_AUTO


def test_config_defaults():
    L = dg.lib()
    cfg = _lib.DycConfig()
    L.dyc_config_default(C.byref(cfg))
    assert (cfg.key_bytes, cfg.value_bytes, cfg.num_subtables, cfg.bucket_bytes) == (4, 4, 4, 128)
    assert cfg.upper_load == 0.8 and cfg.lower_load == 0.5
    assert cfg.min_downsize_capacity == int(4 * 1024 * 1024 * 1.2)
    assert cfg.auto_resize == 1


@pytest.mark.parametrize("field,value", [("key_bytes", 3), ("value_bytes", 2),
                                         ("num_subtables", 7), ("num_subtables", 1),
                                         ("bucket_bytes", 48), ("max_evictions", 0)])
def test_invalid_config_rejected_before_any_device_call(field, value):
    L = dg.lib()
    cfg = _lib.DycConfig()
    L.dyc_config_default(C.byref(cfg))
    setattr(cfg, field, value)
    h = C.c_void_p()
    assert L.dyc_create(C.byref(cfg), C.byref(h)) == _lib.DYC_EINVAL
    assert not h.value
    assert L.dyc_last_error()


def test_null_arguments_rejected():
    L = dg.lib()
    assert L.dyc_insert(None, None, None, 1, 0, None) == _lib.DYC_EINVAL
    assert L.dyc_find(None, None, None, None, 1, None) == _lib.DYC_EINVAL
    assert L.dyc_erase(None, None, 1, None, None, 0, None) == _lib.DYC_EINVAL
    assert L.dyc_destroy(None) == _lib.DYC_OK
    assert L.dyc_apply(None, None, None, None, 1, None, None, 0, None) == _lib.DYC_EINVAL
    assert L.dyc_set_spare_cache(None, 0) == _lib.DYC_EINVAL
    assert L.dyc_set_spare_bytes(None, None) == _lib.DYC_EINVAL
    assert L.dyc_status_string(_lib.DYC_EOVERFLOW) == b"eviction overflow"


def test_four_byte_keys_need_four_byte_values():
    L = dg.lib()
    cfg = _lib.DycConfig()
    L.dyc_config_default(C.byref(cfg))
    cfg.value_bytes = 8
    h = C.c_void_p()
    assert L.dyc_create(C.byref(cfg), C.byref(h)) == _lib.DYC_EINVAL


def test_snapshot_header_layout(tmp_path):
    prog = tmp_path / "snap.c"
    prog.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "dycuckoo.h"\n'
        "int main(void){printf(\"%zu %zu %zu %zu %zu\\n\", sizeof(dyc_snapshot_header),"
        " offsetof(dyc_snapshot_header, size), offsetof(dyc_snapshot_header, nbuckets),"
        " offsetof(dyc_snapshot_header, payload_bytes), offsetof(dyc_snapshot_header, checksum));"
        "return 0;}\n")
    exe = tmp_path / "snap"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(prog), "-o", str(exe)],
                   check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    assert got == [256, 40, 88, 112, 120]


def _snap_header(**over):
    import numpy as np
    h = np.zeros(256, np.uint8)
    h[:8] = np.frombuffer(b"DYCSNAP1", np.uint8)
    u32 = h.view(np.uint32)
    u64 = h.view(np.uint64)
    f64 = h.view(np.float64)
    u32[2], u32[3] = 2, 256
    u32[4:10] = [4, 4, 128, 4, 64, 1]          # widths, bucket, d, bound, auto
    u64[5], u64[6] = 0, 4 * 2 * 15             # size, capacity
    f64[7], f64[8] = 0.8, 0.5
    u64[9], u64[10] = 0, 1024
    u32[22:28] = [2, 2, 2, 2, 0, 0]            # nbuckets
    u64[14] = 4 * 2 * 128                      # payload
    for k, v in over.items():
        {"u32": u32, "u64": u64}[k[:3]][int(k[4:])] = v
    return h


def test_restore_rejects_malformed_snapshots_before_any_device_call():
    import numpy as np
    L = dg.lib()
    h = C.c_void_p()
    good = np.concatenate([_snap_header(), np.zeros(1024, np.uint8)])
    bad = [np.zeros(100, np.uint8),                                   # shorter than a header
           np.concatenate([_snap_header(u32_2=1), np.zeros(1024, np.uint8)]),   # version
           np.concatenate([_snap_header(u32_4=3), np.zeros(1024, np.uint8)]),   # key width
           np.concatenate([_snap_header(u64_14=999), np.zeros(1024, np.uint8)]),  # payload
           np.concatenate([_snap_header(u64_5=10 ** 6), np.zeros(1024, np.uint8)]),  # size > slots
           good[:600]]                                                 # truncated payload
    for i, b in enumerate(bad):
        assert L.dyc_restore(b.ctypes.data, b.size, 0, C.byref(h)) == _lib.DYC_EINVAL, i
        assert not h.value
    wrong_magic = good.copy()
    wrong_magic[0] = ord("X")
    assert L.dyc_restore(wrong_magic.ctypes.data, wrong_magic.size, 0, C.byref(h)) == _lib.DYC_EINVAL
