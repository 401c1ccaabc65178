"""TEST INFRASTRUCTURE ONLY: build the reference's own code for the oracle pin.

Recipe that compiles parts of the reference (pauline-ly/databases_gpu,
GPU/dyhash) from where they lie under /root/reference into oracle/_ref/:

  libref_host.so  host C++ build of the reference's hash functions, pair maps,
                  makeEntry, isPrime/nextPrime, the hashAPI sizing and resize
                  target choice (line ranges of cuckoo.cu, api.cpp and
                  diff_hash_num_pos_fun.cpp wrapped by ref_host_glue.inc), plus
                  mt19937ar.cpp and random_numbers.cpp compiled as they are.
  libref_gpu.so   the reference's GPU kernels (cuckoo.cu as it is: insert,
                  search, delete, resize up/down) for sm_103a with nvcc, behind
                  the C launchers of ref_gpu_glue.cu; the pre-Volta warp
                  intrinsics are mapped to their _sync forms on the calling
                  16-lane group by ref_shim/gpu/ref_warp_sync.h.

Nothing is copied into the repository: the generated translation unit, the
staged sources and the libraries live under oracle/_ref/, which git ignores.
The reference tree only exists in the build container. The host library is
built there (tests/golden/make_golden.py turns its outputs into committed
fixtures). The GPU library has to be built on the GPU machine, which has no
reference tree and cannot run objects built here, so stage_gpu() copies the
handful of reference files cuckoo.cu needs into oracle/_ref/src/ (ignored
like the rest of oracle/_ref/, and carried to the GPU machine with it), and
build_gpu() compiles from there wherever it runs.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("DYC_REFERENCE_ROOT", "/root/reference")
DYHASH = os.path.join(REF_ROOT, "GPU", "dyhash")
OUT = os.path.join(HERE, "_ref")
BUILD = os.path.join(OUT, "build")
CUDA_INC = "/usr/local/cuda/include"


def available() -> bool:
    return os.path.isfile(os.path.join(DYHASH, "cuckoo.cu"))


def _lines(path: str, lo: int, hi: int) -> str:
    with open(path, encoding="utf-8", errors="replace") as f:
        src = f.read().split("\n")
    name = os.path.relpath(path, REF_ROOT)
    return '#line %d "%s"\n' % (lo, name) + "\n".join(src[lo - 1:hi]) + "\n"


def _generate() -> str:
    cu = os.path.join(DYHASH, "cuckoo.cu")
    api = os.path.join(DYHASH, "api.cpp")
    var = os.path.join(DYHASH, "diff_hash_num_pos_fun.cpp")
    parts = [
        "// generated by oracle/build_ref.py from the reference tree; not committed\n",
        '#include "cuckoo.h"\n',
        _lines(cu, 16, 18),     # __constant__ table, get_table_length
        _lines(cu, 27, 64),     # get_hash1..4
        _lines(cu, 76, 90),     # hash_function
        _lines(cu, 110, 120),   # get_hash5
        "namespace dyc_ref_d4 {\n", _lines(cu, 190, 213), _lines(cu, 310, 313), "}\n",
        "namespace dyc_ref_d2 {\n", _lines(var, 16, 29), "}\n",
        "namespace dyc_ref_d3 {\n", _lines(var, 38, 55), "}\n",
        "namespace dyc_ref_d5 {\n", _lines(var, 120, 146), "}\n",
        _lines(api, 4, 22),     # isPrime, nextPrime
        'extern "C" uint32_t ref_subtable_buckets(TYPE size) {\n',
        _lines(api, 47, 51), "    return s_bucket;\n}\n",
        'extern "C" uint32_t ref_pick_up(const uint32_t *lsize) {\n'
        "    cuckoo tmp; cuckoo *h_table = &tmp;\n"
        "    for (int i = 0; i < TABLE_NUM; ++i) tmp.Lsize[i] = lsize[i];\n",
        _lines(api, 116, 122), "    return num_table_to_resize;\n}\n",
        'extern "C" uint32_t ref_pick_down(const uint32_t *lsize) {\n'
        "    cuckoo tmp; cuckoo *h_table = &tmp;\n"
        "    for (int i = 0; i < TABLE_NUM; ++i) tmp.Lsize[i] = lsize[i];\n",
        _lines(api, 147, 153), "    return num_table_to_resize;\n}\n",
        '#include "%s"\n' % os.path.join(HERE, "ref_host_glue.inc"),
    ]
    os.makedirs(BUILD, exist_ok=True)
    path = os.path.join(BUILD, "ref_host.cpp")
    with open(path, "w") as f:
        f.write("".join(parts))
    return path


def build() -> str | None:
    """Build oracle/_ref/libref_host.so and stage and build the GPU library;
    returns the host library's path or None without a reference tree."""
    if not available():
        return None
    os.makedirs(os.path.join(BUILD, "inc", "x"), exist_ok=True)
    # dy_hash.h includes "../test_uilt.h" relative to a search directory.
    with open(os.path.join(BUILD, "inc", "test_uilt.h"), "w") as f:
        f.write('#include "%s"\n' % os.path.join(DYHASH, "test_uilt.h"))
    tu = _generate()
    lib = os.path.join(OUT, "libref_host.so")
    cmd = [
        "g++", "-std=c++14", "-O2", "-fPIC", "-shared", "-w",
        "-I", os.path.join(HERE, "ref_shim", "host"),
        "-I", os.path.join(HERE, "ref_shim", "common"),
        "-I", os.path.join(BUILD, "inc", "x"),
        "-I", DYHASH, "-I", CUDA_INC,
        "-o", lib, tu,
        os.path.join(DYHASH, "mt19937ar.cpp"),
        os.path.join(DYHASH, "random_numbers.cpp"),
    ]
    subprocess.check_call(cmd)
    stage_gpu()
    build_gpu()
    return lib


# ---------------------------------------------------------------- GPU kernels
# The files cuckoo.cu includes (directly or through api.h / cuckoo.h /
# dy_hash.h); dy_hash.h reaches test_uilt.h as "../test_uilt.h".
GPU_FILES = ["cuckoo.cu", "cuckoo.h", "api.h", "dy_hash.h", "gputimer.h", "cnmem.h",
             "random_numbers.h"]
STAGE = os.path.join(OUT, "src")
STAGE_DYHASH = os.path.join(STAGE, "dyhash")
GPU_LIB = os.path.join(OUT, "libref_gpu.so")
GPU_GLUE = os.path.join(HERE, "ref_gpu_glue.cu")
GPU_SHIM = os.path.join(HERE, "ref_shim", "gpu", "ref_warp_sync.h")


def stage_gpu() -> bool:
    """Copy the reference files the GPU build needs into oracle/_ref/src/
    (only where the reference tree is present); True when staged."""
    if not available():
        return gpu_staged()
    import shutil
    os.makedirs(STAGE_DYHASH, exist_ok=True)
    for f in GPU_FILES:
        src, dst = os.path.join(DYHASH, f), os.path.join(STAGE_DYHASH, f)
        if not os.path.exists(dst) or os.path.getmtime(dst) < os.path.getmtime(src):
            shutil.copyfile(src, dst)
    dst = os.path.join(STAGE, "test_uilt.h")
    if not os.path.exists(dst):
        shutil.copyfile(os.path.join(DYHASH, "test_uilt.h"), dst)
    return True


def gpu_staged() -> bool:
    return all(os.path.isfile(os.path.join(STAGE_DYHASH, f)) for f in GPU_FILES) and \
        os.path.isfile(os.path.join(STAGE, "test_uilt.h"))


def _nvcc() -> str:
    import shutil
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def build_gpu(force: bool = False) -> str | None:
    """Compile oracle/_ref/libref_gpu.so from the staged reference source;
    None when nothing is staged."""
    if not gpu_staged():
        return None
    inputs = [GPU_GLUE, GPU_SHIM] + [os.path.join(STAGE_DYHASH, f) for f in GPU_FILES]
    if not force and os.path.exists(GPU_LIB) and \
            all(os.path.getmtime(f) <= os.path.getmtime(GPU_LIB) for f in inputs):
        return GPU_LIB
    tmp = GPU_LIB + ".tmp%d" % os.getpid()
    cmd = [_nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo",
           "-std=c++14", "-shared", "-Xcompiler", "-fPIC", "-w", "-cudart", "shared",
           "-include", GPU_SHIM,
           "-I", os.path.join(HERE, "ref_shim", "common"), "-I", STAGE_DYHASH,
           "-o", tmp, GPU_GLUE]
    subprocess.check_call(cmd)
    os.replace(tmp, GPU_LIB)
    return GPU_LIB


if __name__ == "__main__":
    p = build()
    print(p if p else "reference tree not present; nothing built")
    sys.exit(0)
