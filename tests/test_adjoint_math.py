"""The adjoint's derivative code on the host: element-local vector-Jacobian
products (lg_adjoint_math.h) against central finite differences of the
forward formulas, for random elements, every branch of the limiter and both
signs of the volume change in the EOS; whole cycles (lg_adjoint_cycle.h)
against branch-replayed differences of the oracle, for the terminal-energy
objective and for seeds on every carried field."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_element_vjps_match_finite_differences(tmp_path):
    if not shutil.which("g++"):
        pytest.skip("no host C++ compiler")
    exe = tmp_path / "adjoint_selftest"
    subprocess.run(["g++", "-O1", "-std=c++17", "-I", os.path.join(ROOT, "lulesh_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "adjoint_selftest.cc"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    worst = float(r.stdout.strip().splitlines()[-1].split()[-1])
    assert r.returncode == 0 and worst < 1e-6, r.stdout[-2000:]


def test_whole_cycle_adjoint_matches_finite_differences(tmp_path):
    """lg_adjoint_cycle.h's item functions -- the GPU adjoint kernels' code --
    looped on the host over oracle states, against central differences of
    the oracle replaying the forward run's branch decisions (decision tape):
    three single-element probes, three random directions over the noisy
    elements, and hgcoef, on three meshes."""
    if not shutil.which("g++") or not shutil.which("gcc"):
        pytest.skip("no host compilers")
    obj = tmp_path / "orc.o"
    exe = tmp_path / "adjoint_cycle_selftest"
    subprocess.run(["gcc", "-O1", "-std=c11", "-ffp-contract=off", "-DORC_TAPE", "-c",
                    os.path.join(ROOT, "oracle", "lulesh_oracle.c"), "-o", str(obj)], check=True)
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "lulesh_gb300", "csrc"),
                    "-I", os.path.join(ROOT, "oracle"),
                    os.path.join(ROOT, "tests", "adjoint_cycle_selftest.cc"), str(obj), "-o",
                    str(exe)], check=True)
    # each check must agree at relative step 1e-6 or 1e-7: the larger step
    # carries truncation error on these small noisy meshes, the smaller one
    # round-off
    best = {}
    for rel in ("1e-6", "1e-7"):
        env = dict(os.environ, LG_FD_REL=rel, LG_FD_BRANCH="1")
        for args in (["6", "5", "216"], ["12", "40", "40"], ["20", "60", "200"]):
            r = subprocess.run([str(exe)] + args, capture_output=True, text=True, env=env)
            assert r.returncode == 0, r.stdout + r.stderr
            for line in r.stdout.splitlines():
                if line.startswith(("e0 dir", "hgcoef")):
                    key = (tuple(args), line.split(":")[0])
                    best[key] = min(best.get(key, 1.0), float(line.split()[-1]))
    assert len(best) == 21 and max(best.values()) < 1e-6, best


def test_general_vjp_matches_finite_differences_in_mid_run(tmp_path):
    """The reverse-mode product for a seed on every carried field, from a
    state some cycles into a run whose every node moves: each initial field's
    directional derivative and dJ/dhgcoef against branch-replayed central
    differences (Richardson).  The oracle here is double precision, so the
    differences carry ~1e-6 of round-off; the GPU test checks the same product
    against the long double oracle to 1e-14."""
    if not shutil.which("g++") or not shutil.which("gcc"):
        pytest.skip("no host compilers")
    obj = tmp_path / "orc.o"
    exe = tmp_path / "adjoint_vjp_selftest"
    subprocess.run(["gcc", "-O1", "-std=c11", "-ffp-contract=off", "-DORC_TAPE", "-c",
                    os.path.join(ROOT, "oracle", "lulesh_oracle.c"), "-o", str(obj)], check=True)
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "lulesh_gb300", "csrc"),
                    "-I", os.path.join(ROOT, "oracle"),
                    os.path.join(ROOT, "tests", "adjoint_vjp_selftest.cc"), str(obj), "-o",
                    str(exe)], check=True)
    best = {}
    for rel in ("1e-6", "1e-7"):
        env = dict(os.environ, LG_FD_REL=rel)
        for args in (["6", "2", "6"], ["6", "5", "8"], ["10", "8", "16"]):
            r = subprocess.run([str(exe)] + args, capture_output=True, text=True, env=env)
            assert r.returncode == 0, r.stdout + r.stderr
            for line in r.stdout.splitlines()[:-1]:
                key = (tuple(args), line.split()[0])
                best[key] = min(best.get(key, 1.0), float(line.split()[-1]))
    assert len(best) == 36 and max(best.values()) < 1e-5, best
