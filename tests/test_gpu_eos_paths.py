"""The EOS's unit-density path (refdens == 1: the sound-speed terms skip
x / refdens) against its general path, on elements at rest, compressing and
expanding (tests/eos_paths_selftest.cu, built with nvcc and run on the GPU):
bit for bit without contraction, within 1e-13 with it."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("strict", [True, False], ids=["fp64", "fp64-fma"])
def test_unit_density_path_matches_general(native_lib, tmp_path, strict):
    from lulesh_gb300 import build
    exe = tmp_path / "eos_paths_selftest"
    flags = ["--fmad=false", "-DEOS_SELFTEST_STRICT=1"] if strict else ["--fmad=true"]
    subprocess.run([build._nvcc()] + build.ARCH + ["-O3", "-std=c++17"] + flags +
                   ["-I", os.path.join(ROOT, "lulesh_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "eos_paths_selftest.cu"), "-o", str(exe)],
                   check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    if strict:
        assert "differing 0," in r.stdout
