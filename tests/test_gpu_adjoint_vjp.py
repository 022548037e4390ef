"""The general reverse-mode product of the cycles (lg_adjoint_vjp).

For an objective J(final state) the caller seeds dJ/d(final field) for any of
the carried fields (x y z xd yd zd e p q v ss) and receives dJ/d(initial
field) for all of them and dJ/dhgcoef.  Checked: it reproduces lg_adjoint
for the terminal-energy seed, it is linear in the seed, and every initial
field's gradient agrees with central differences of the oracle replaying the
base run's branch decisions in extended precision (orc_tape_replay,
Richardson over two steps) -- the same check the s=48 study uses, here on a
small noisy problem and for all eleven fields.
"""
import numpy as np
import pytest

import adjoint_case as case

pytestmark = pytest.mark.gpu
FIELDS = ["x", "y", "z", "xd", "yd", "zd", "e", "p", "q", "v", "ss"]
NODE = {"x", "y", "z", "xd", "yd", "zd"}


def _problem(nx=10, ncycles=30, nnoise=120):
    import lulesh_gb300 as lg
    from lulesh_gb300.autograd import TerminalEnergyProblem
    e_setup = lg.Domain(nx, 11, device=-1).field("e")
    e_noisy, _ = case.initial_energy(e_setup, nx, nnoise)
    return TerminalEnergyProblem(nx, 11, ncycles, 7, e_base=e_noisy), e_noisy


def test_vjp_reproduces_terminal_energy_adjoint(native_lib):
    pr, e0 = _problem()
    J, ge, gh = pr.value_and_grad(e0, pr.hg_base)
    volo = pr.dom.field("volo")
    grads, gh2 = pr.vjp(e0, pr.hg_base, {"e": np.where(pr.mask, volo, 0.0)}, want=FIELDS)
    assert np.array_equal(grads["e"], ge) and gh2 == gh
    assert set(grads) == set(FIELDS)


def test_vjp_is_linear_in_the_seed(native_lib):
    pr, e0 = _problem()
    rng = np.random.default_rng(1)
    E, N = pr.dom.numElem, pr.dom.numNode
    s1 = {"e": rng.standard_normal(E), "xd": rng.standard_normal(N)}
    s2 = {"p": rng.standard_normal(E), "x": rng.standard_normal(N)}
    g1, h1 = pr.vjp(e0, pr.hg_base, s1, want=FIELDS)
    g2, h2 = pr.vjp(e0, pr.hg_base, s2, want=FIELDS)
    both = {**{k: 2.0 * v for k, v in s1.items()}, **{k: -3.0 * v for k, v in s2.items()}}
    g, h = pr.vjp(e0, pr.hg_base, both, want=FIELDS)
    for f in FIELDS:
        ref = 2.0 * g1[f] - 3.0 * g2[f]
        scale = max(np.abs(ref).max(), 1e-300)
        assert np.abs(g[f] - ref).max() <= 1e-12 * scale, f
    assert abs(h - (2.0 * h1 - 3.0 * h2)) <= 1e-12 * max(abs(h), 1e-300)


def test_vjp_every_field_against_branch_replay(native_lib, oracle_built, capsys):
    """J = sum over fields of seed_f . final_f with random seeds; for each
    initial field a random perturbation direction; the adjoint's directional
    derivative against the extended-precision branch replay.

    The state differentiated at is a few cycles into a run whose every
    element holds energy, so that every node but the origin moves.  At rest
    the Q limiter's gradient ratios are 0/0: q then grows like
    |dv| (1 - phi(direction)), which has directional derivatives but no
    gradient with respect to velocities, pressures or viscosities.  (The first
    cycle from the set-up is such a state: p = 0 until its EOS, so no force
    moves a node before the element phase.)"""
    import lulesh_gb300 as lg
    from oracle.oracle import OracleDomain
    nx, npre, ncyc = 6, 5, 8
    e_setup = lg.Domain(nx, 11, device=-1).field("e")
    e0 = e_setup + 1e-3 * e_setup[0] * (1.0 + np.random.default_rng(5).random(e_setup.size))
    dom = lg.Domain(nx, 11, its=10 ** 9)
    dom.set_field("e", e0)
    dom.dt_record(npre + ncyc)
    assert dom.step(npre + ncyc) == 0
    dts = dom.dt_get(npre + ncyc)
    dom.dt_record(0)
    dom.dt_freeze(dts)
    dom.reset()
    dom.set_field("e", e0)
    assert dom.step(npre) == 0
    base = {f: dom.field(f) for f in FIELDS}
    speed = np.abs(base["xd"]) + np.abs(base["yd"]) + np.abs(base["zd"])
    assert np.array_equal(np.flatnonzero(speed == 0), [0])
    E, N = dom.numElem, dom.numNode
    rng = np.random.default_rng(3)
    seeds = {f: rng.standard_normal(N if f in NODE else E) for f in FIELDS}
    grads, gh = dom.adjoint_vjp(ncyc, seeds, FIELDS, ckpt=3)

    def run(state, src=None, record=False):
        o = OracleDomain(nx, 11, extended=True)
        o.dt_freeze(dts)
        o.set_scalar("cycle", npre)
        for f in FIELDS:
            o.field(f)[:] = state[f]
        if record:
            o.tape_record(ncyc)
        if src is not None:
            o.tape_replay(src)
        assert o.step(ncyc) == 0
        J = sum(np.dot(seeds[f].astype(np.longdouble), o.field(f)) for f in FIELDS)
        return J, o

    _, rec = run({f: base[f].astype(np.longdouble) for f in FIELDS}, record=True)
    # each direction scaled by its field's size in this state; Richardson over
    # relative steps 1e-6 and 1e-7 (the replay is smooth there: steps 1e-7 and
    # 1e-8 give the same extrapolation to 1e-8)
    errs = {}
    for f in FIELDS:
        d = rng.standard_normal(N if f in NODE else E) * max(np.abs(base[f]).max(), 1e-3)
        ad = float(np.dot(grads[f], d))
        fds = []
        for h in (1e-6, 1e-7):
            plus = {g: base[g].astype(np.longdouble) for g in FIELDS}
            minus = {g: base[g].astype(np.longdouble) for g in FIELDS}
            plus[f] = plus[f] + np.longdouble(h) * d
            minus[f] = minus[f] - np.longdouble(h) * d
            fds.append(float((run(plus, rec)[0] - run(minus, rec)[0]) / (2 * np.longdouble(h))))
        fd = fds[1] + (fds[1] - fds[0]) / 99
        errs[f] = abs(ad - fd) / max(abs(fd), 1e-300)
    with capsys.disabled():
        print("\nVJP vs branch replay, per initial field: "
              + " ".join(f"{f}={v:.1e}" for f, v in errs.items()))
    assert max(errs.values()) <= 1e-6, errs


def test_final_energy_field_autograd(native_lib):
    """A torch loss of FinalEnergyField's output backpropagates through
    lg_adjoint_vjp: for the masked terminal energy as the loss it gives
    TerminalEnergy's gradients exactly; for a quadratic loss it gives the VJP
    of that loss's own gradient."""
    import torch
    from lulesh_gb300.autograd import FinalEnergyField, TerminalEnergy
    pr, e0 = _problem()
    volo = torch.from_numpy(pr.dom.field("volo"))
    mask = torch.from_numpy(pr.mask.astype(np.float64))

    e0a = torch.tensor(e0, requires_grad=True)
    hga = torch.tensor(pr.hg_base, dtype=torch.float64, requires_grad=True)
    ef = FinalEnergyField.apply(e0a, hga, pr)
    (ef * volo * mask).sum().backward()

    e0b = torch.tensor(e0, requires_grad=True)
    hgb = torch.tensor(pr.hg_base, dtype=torch.float64, requires_grad=True)
    TerminalEnergy.apply(e0b, hgb, pr).backward()
    assert torch.equal(e0a.grad, e0b.grad) and torch.equal(hga.grad, hgb.grad)

    e0c = torch.tensor(e0, requires_grad=True)
    ef = FinalEnergyField.apply(e0c, torch.tensor(pr.hg_base, dtype=torch.float64), pr)
    target = ef.detach() * 0.9
    ((ef - target) ** 2).sum().backward()
    seed = 2.0 * (ef.detach() - target).numpy()
    grads, _ = pr.vjp(e0, pr.hg_base, {"e": seed}, want=("e",))
    assert np.array_equal(e0c.grad.numpy(), grads["e"])
