"""Float-float arithmetic of the mixed mode's recurrences (edgpu_internal.cuh: ffloat), checked on the host:
tests/cpp/ffloat_check.cu is compiled as host code by nvcc and compares sums, products, 16-term
multiply-accumulate chains and cancellations with long-double references on seeded random operands."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    return None


def test_float_float_arithmetic_error_bounds(tmp_path):
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "ffloat_check")
    src = os.path.join(HERE, "cpp", "ffloat_check.cu")
    r = subprocess.run([nvcc, "-std=c++17", "-O2", "-o", exe, src], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
