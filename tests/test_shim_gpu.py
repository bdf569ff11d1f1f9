"""The drop-in C++ header (include/rsort/rsort.cuh) used the way rsort's own
examples use it, compiled against libgbsort.so (tests/cpp/rsort_shim_test.cpp)."""

import os
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIN = os.path.join(REPO, "cuda-fast-sort_gb300", "_build", "rsort_shim_test")


def test_shim_header_compiles_on_host():
    """The header needs only cuda_runtime_api.h and gbsort.h (no device code)."""
    src = '#include "rsort/rsort.cuh"\nint main(){ size_t t=0; float* k=nullptr;\n' \
          'rsort::sort(k, &t, (uint8_t*)nullptr, 100); return t ? 0 : 1; }\n'
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-x", "c++", "-", "-I", os.path.join(REPO, "include"),
                        "-I", "/usr/local/cuda/include"], input=src, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_shim_program_on_gpu(cuda):
    assert os.path.exists(BIN), "build() compiles the shim test"
    r = subprocess.run([BIN], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL PASSED" in r.stdout
