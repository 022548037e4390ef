"""Host checks of the exactness claims the FP64 kernels rest on.

1. lg_geometry.cuh applies the reference's power-of-two factors once (face
   areas, Jacobian, half-step B matrix, monotonic-Q gradients).  Compiled for
   the host without contraction it must give the oracle's bits on random
   hexahedra and on a jittered mesh (geometry_selftest.cc against the oracle's
   own functions through geometry_ref_shim.c).
2. The kernels compare doubles on the integer pipe through an
   order-preserving key (dkey in lg_cycle_common.cuh, lt in lg_geometry.cuh):
   key = (b ^ (sign & 0x7fff...)) - sign, sign = b >> 63.  Restated here in
   int64 arithmetic, it must order every non-NaN double as IEEE comparison
   does, with -0 equal to +0.
3. The nodal acceleration f / m is formed from the constant RN(1/m) by
   Markstein's residual correction (div_by_mass in lg_kernels.cuh); restated
   in division_selftest.cc, it must equal the IEEE quotient.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def geometry_selftest(tmp_path_factory):
    if not shutil.which("g++") or not shutil.which("gcc"):
        pytest.skip("no host compilers")
    tmp = tmp_path_factory.mktemp("geometry")
    shim = tmp / "shim.o"
    exe = tmp / "geometry_selftest"
    subprocess.run(["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-I", os.path.join(ROOT, "oracle"),
                    "-c", os.path.join(ROOT, "tests", "geometry_ref_shim.c"), "-o", str(shim)],
                   check=True)
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                    "-I", os.path.join(ROOT, "lulesh_gb300", "csrc"), "-I", os.path.join(ROOT, "oracle"),
                    os.path.join(ROOT, "tests", "geometry_selftest.cc"), str(shim), "-lm",
                    "-o", str(exe)], check=True)
    return str(exe)


def test_folded_geometry_equals_oracle_bitwise(geometry_selftest):
    r = subprocess.run([geometry_selftest, "100000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout[-2000:]
    assert r.stdout.strip().endswith("mismatches 0"), r.stdout[-2000:]


# every reassociated form the FMA build uses, by the label of its check
REASSOCIATED = ["normal x from diagonals", "normal y from diagonals", "normal z from diagonals",
                "char_length from diagonals", "volume gradient x", "volume gradient y",
                "volume gradient z", "dxx from diagonals", "dyy from diagonals",
                "dzz from diagonals", "velocity trace from directions", "delx from diagonals",
                "delv from diagonals"]


def test_reassociated_tolerances_see_a_planted_error(geometry_selftest):
    """The oracle's values scaled by 1 + 1e-8 (plant mode): each reassociated
    form's tolerance is tight enough that its check reports elements beyond it."""
    r = subprocess.run([geometry_selftest, "20000", "plant"], capture_output=True, text=True)
    assert r.returncode == 1, r.stdout[-2000:]
    tripped = {}
    for line in r.stdout.splitlines():
        if line.startswith("planted "):
            label, rest = line[len("planted "):].rsplit(": ", 1)
            tripped[label] = int(rest.split()[0])
    for label in REASSOCIATED:
        assert tripped.get(label, 0) > 0, (label, tripped)


def _dkey(v: np.ndarray) -> np.ndarray:
    b = v.view(np.int64)
    sign = b >> 63
    return (b ^ (sign & np.int64(0x7FFFFFFFFFFFFFFF))) - sign


def test_integer_key_orders_doubles_like_ieee():
    rng = np.random.default_rng(7)
    special = np.array([0.0, -0.0, 1e-308, -1e-308, 5e-324, -5e-324, 2.2250738585072014e-308,
                        1.0, -1.0, 1e308, -1e308, np.inf, -np.inf, 1e-36, -1e-36, 1e-7, -1e-7,
                        -1e15, 1e20, 1.111111e-37, 3.333333e-19])
    mags = 10.0 ** rng.uniform(-310, 308, 20000)
    rand = np.concatenate([mags, -mags, rng.standard_normal(20000),
                           np.nextafter(special, np.inf), np.nextafter(special, -np.inf)])
    vals = np.concatenate([special, rand]).astype(np.float64)
    a = np.repeat(vals[:600], 600)
    b = np.tile(vals[:600], 600)
    ka, kb = _dkey(a), _dkey(b)
    assert np.array_equal(ka < kb, a < b)
    assert np.array_equal(ka <= kb, a <= b)
    a, b = rng.permutation(vals), rng.permutation(vals)
    ka, kb = _dkey(a), _dkey(b)
    assert np.array_equal(ka < kb, a < b)
    assert np.array_equal(ka <= kb, a <= b)
    # |a| < c on the magnitude bits, for c >= +0
    cuts = np.array([0.0, 1e-7, 1e-36, 1.0, np.inf])
    mag = np.abs(a).view(np.int64)
    for c in cuts:
        assert np.array_equal(mag < np.float64(c).view(np.int64), np.abs(a) < c)


def test_mass_quotient_equals_ieee_division(tmp_path):
    if not shutil.which("g++"):
        pytest.skip("no host C++ compiler")
    exe = tmp_path / "division_selftest"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                    os.path.join(ROOT, "tests", "division_selftest.cc"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe), "20000000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout[-2000:]
    assert r.stdout.strip().endswith("mismatches 0"), r.stdout[-2000:]
