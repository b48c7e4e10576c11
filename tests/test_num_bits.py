"""
The FP64 kernels (standard loop, FP64 and Xrange perturbation) replace some
double operations by tests on the bit patterns (fsg_num.cuh: zero and
magnitude tests, the escape and stationarity compares, the product of a real
by a complex without its products with zero).  They must give the bits of
the operations they stand for: the device header is compiled for the host
and checked against the double operations on random and special operands
(signed zeros, subnormals, infinities, NaNs of both signs).
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _cuda_include():
    for root in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if root and os.path.exists(os.path.join(root, "include", "cuda_runtime.h")):
            return os.path.join(root, "include")
    return None


def test_bit_pattern_helpers_match_double_operations(tmp_path):
    cxx = shutil.which("g++")
    inc = _cuda_include()
    if cxx is None or inc is None:
        pytest.skip("g++ or the CUDA headers are missing")
    exe = str(tmp_path / "num_bits_check")
    src = os.path.join(HERE, "native", "num_bits_check.cpp")
    r = subprocess.run([cxx, "-O0", "-ffp-contract=off", "-std=c++17", "-I", inc, src, "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([exe, "1000000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 mismatches" in r.stdout
