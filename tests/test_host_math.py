"""Host-side checks of two pieces of arithmetic the device kernels rely on, built from the
library's own headers (nvcc, host code only, no GPU):

* radix_plan (fft.cuh): every transform length up to 1024 is factored into supported stages whose
  product is the length, with consistent stage divisors; 7-smooth lengths use register radices
  only and few stages; known plans of the padded extents.
* make_fastdiv (common.hpp): the constants of the 32-bit division q = (umulhi(n, m) + n) >> l give
  floor(n / d) for every divisor up to 4096 over dense and near-multiple dividends and for large
  divisors at the edges of the int range (the kernels divide non-negative ints only).
"""
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _nvcc():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return os.path.join(c, "bin", "nvcc")
    return shutil.which("nvcc")


def test_radix_plan_and_fastdiv():
    nvcc = _nvcc()
    if not nvcc:
        pytest.skip("nvcc not found")
    exe = os.path.join(tempfile.mkdtemp(), "plan_check")
    src = os.path.join(ROOT, "tests", "hostcheck", "plan_check.cu")
    r = subprocess.run([nvcc, "-std=c++17", "-O2", "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "spirit_gb300", "csrc"),
                        src, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout[-3000:]
