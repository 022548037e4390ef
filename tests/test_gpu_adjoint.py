"""Checkpointed adjoint (lg_adjoint) against central finite differences.

J = total internal energy sum(e * volo) of the elements whose centroid lies
within r = 0.5 of the origin after the last cycle; the time-step sequence is
frozen from the forward run of the noisy initial field (tests/adjoint_case.py).
Gradients with respect to the initial energy field (16 seeded directions) and
hgcoef are compared with central differences of the plain GPU path and, at
the full size, with central differences of the oracle replaying the base
run's branch decisions and of the reference CPU build
(tests/golden/make_adjoint_fd.py).  Bar: 1e-6 relative.
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
    assert float(J.detach()) == Jr
    assert np.array_equal(e.grad.numpy(), ge) and float(hg.grad) == gh


def test_adjoint_s48_200_cycles(native_lib, capsys):
    """The full study: s=48, 200 cycles, checkpoint every 20, on the time
    steps and mask of the fixture's oracle run.

    Over 200 cycles the noisy field drives delvc through zero in elements
    whose monotonic-Q terms are nonzero, so J itself jumps (lulesh.cc:
    2079-2081, 2122-2124) many times within one finite-difference step, in
    the reference build as in this path; plain central differences of the
    two agree with each other, not with any derivative.  The adjoint is
    checked against central differences of the oracle replaying the branch
    decisions of the base run (orc_tape_replay), which is smooth there;
    elements crossing zero energy put square roots of near-zero arguments
    on that branch, so its differences converge (as h^2) only below relative
    step 1e-8, where double-precision round-off of J (~2e-13) already costs
    1e-6..1e-5 of the smaller derivatives.  The check of record is the
    replay in long double (2,000x less round-off) at steps 1e-9 and 1e-10,
    Richardson-extrapolated."""
    if not os.path.exists(GOLDEN):
        pytest.skip("adjoint fixture not generated (tests/golden/make_adjoint_fd.py)")
    g = json.load(open(GOLDEN))
    from lulesh_gb300.autograd import TerminalEnergyProblem
    import lulesh_gb300 as lg
    e_setup = lg.Domain(case.NX, case.NREG, device=-1).field("e")
    e_noisy, idx = case.initial_energy(e_setup, case.NX)
    mask = np.zeros(case.NX ** 3, bool)
    mask[g["mask_idx"]] = True
    pr = TerminalEnergyProblem(case.NX, case.NREG, case.NCYCLES, case.CKPT, e_base=e_noisy,
                               dts=np.array(g["dts"]), mask=mask)
    Jf = pr.objective(e_noisy, pr.hg_base)
    t_fwd = t_adj = float("inf")
    for _ in range(3):
        t0 = time.perf_counter()
        pr.objective(e_noisy, pr.hg_base)
        t_fwd = min(t_fwd, time.perf_counter() - t0)
        t0 = time.perf_counter()
        J, ge, gh = pr.value_and_grad(e_noisy, pr.hg_base)
        t_adj = min(t_adj, time.perf_counter() - t0)
    dirs = case.directions(idx, e_noisy)
    ad = [float(ge @ d) for d in dirs] + [gh * case.REL_STEP * pr.hg_base]

    def along(tab, rel):
        """a fixture table as derivatives along the step-1e-6 directions"""
        k = rel / case.REL_STEP
        return [None if f is None else f / k for f in tab["e0"]] + [
            None if tab["hgcoef"] is None else tab["hgcoef"] * case.REL_STEP * pr.hg_base]

    def errs(fd):
        return [None if f is None else abs(a - f) / abs(f) for a, f in zip(ad, fd)]

    steps = {r: along(t, float(r)) for r, t in g["branch_fd"].items()}
    ext = {r: along(t, float(r)) for r, t in g["branch_fd_extended"].items()}

    def richardson(coarse, fine):
        # central differences at h and h/10 with an O(h^2) error:
        # D = D(h/10) + (D(h/10) - D(h)) / 99
        return [None if a is None or b is None else b + (b - a) / 99 for a, b in zip(coarse, fine)]

    rich = richardson(steps["1e-08"], steps["1e-09"])
    rich_ext = richardson(ext["1e-09"], ext["1e-10"])
    plain_ref = errs(along(g["plain_fd_ref"]["1e-06"], 1e-6))
    # this path's own plain central differences at relative step 1e-6
    fd_gpu = [(pr.objective(e_noisy + d, pr.hg_base) - pr.objective(e_noisy - d, pr.hg_base)) / 2
              for d in dirs]
    fd_ref = g["plain_fd_ref"]["1e-06"]["e0"]
    scale = max(abs(f) for f in fd_ref)
    plain_vs_ref = max(abs(a - b) for a, b in zip(fd_gpu, fd_ref)) / scale
    fmt = lambda v: " ".join("  -    " if x is None else f"{x:.1e}" for x in v)  # noqa: E731
    with capsys.disabled():
        print(f"\nadjoint s=48/200: J={J:.12e} (oracle {g['J_oracle']:.12e}, reference "
              f"{g['J_ref']:.12e}) dJ/dhg={gh:.6e} adjoint/forward time {t_adj / t_fwd:.2f}")
        print("  relative error of the adjoint's 16 directional derivatives and dJ/dhgcoef")
        for r, fd in steps.items():
            print(f"  vs branch-replay FD, step {r}: " + fmt(errs(fd)))
        print("  vs branch-replay FD, Richardson 1e-8/1e-9: " + fmt(errs(rich)))
        for r, fd in ext.items():
            print(f"  vs extended-precision branch-replay FD, step {r}: " + fmt(errs(fd)))
        print("  vs extended-precision branch-replay FD, Richardson 1e-9/1e-10: "
              + fmt(errs(rich_ext)))
        print("  vs reference plain FD, step 1e-6: " + fmt(plain_ref))
        print(f"  plain FD of this path vs the reference build's: {plain_vs_ref:.1e} "
              "(of the largest)")
    assert abs(J / Jf - 1) <= 1e-12
    assert abs(J / g["J_ref"] - 1) <= 1e-10 and abs(J / g["J_oracle"] - 1) <= 1e-10
    assert t_adj <= 4 * t_fwd
    # every directional derivative agrees with the extended-precision replay
    # differences to 1e-6
    checked = errs(rich_ext)
    assert None not in checked and max(checked) <= TOL, checked
    # the forward path differentiates like the reference build
    assert plain_vs_ref <= 1e-6
