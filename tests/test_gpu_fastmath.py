"""The mixed path's integer-pipe conversions (lg_fastmath.cuh) against the
hardware's own: to_f32 rounds to nearest, ties to even, like
__double2float_rn for every input that is zero or at least the smallest
normal float, and to_f64 widens exactly (tests/fastmath_selftest.cu, built with nvcc and run on the
GPU)."""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_conversions_match_hardware(native_lib, tmp_path):
    from lulesh_gb300 import build
    nvcc = build._nvcc()
    exe = tmp_path / "fastmath_selftest"
    subprocess.run([nvcc] + build.ARCH + ["-O2", "-std=c++17", "-I",
                                          os.path.join(ROOT, "lulesh_gb300", "csrc"),
                                          os.path.join(ROOT, "tests", "fastmath_selftest.cu"),
                                          "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "to_f32 mismatches 0, to_f64 mismatches 0" in r.stdout
