"""Builds tests/cpp/hashapi_test.cpp -- the reference's gtest cases written
against the C++ hashAPI facade (include/dycuckoo_hashapi.hpp) -- and runs it
on the GPU. Compiling it also runs on the CPU, so the facade always builds."""
import os
import subprocess

import pytest

import databases_gpu_gb300 as dg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = "/usr/local/cuda"


def build_driver(out_dir: str) -> str:
    dg.lib()  # builds libdycuckoo.so if needed
    lib_dir = os.path.dirname(dg.library_path())
    orc = os.path.join(out_dir, "dyc_oracle.o")
    subprocess.run(["gcc", "-O2", "-std=c11", "-c", os.path.join(ROOT, "oracle", "dyc_oracle.c"),
                    "-o", orc], check=True)
    exe = os.path.join(out_dir, "hashapi_test")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(ROOT, "oracle"), "-I", os.path.join(CUDA, "include"),
                    os.path.join(ROOT, "tests", "cpp", "hashapi_test.cpp"), orc,
                    "-L", lib_dir, "-ldycuckoo", "-Wl,-rpath," + lib_dir,
                    "-L", os.path.join(CUDA, "lib64"), "-lcudart", "-lpthread", "-o", exe],
                   check=True)
    return exe


def test_facade_compiles(tmp_path):
    assert os.path.exists(build_driver(str(tmp_path)))


@pytest.mark.gpu
def test_reference_gtest_cases_on_gpu(tmp_path):
    exe = build_driver(str(tmp_path))
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL PASSED" in r.stdout
