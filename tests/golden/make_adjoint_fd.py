"""Generate the adjoint study's finite-difference fixture (adjoint_fd_s48.json).

Run where the reference sources exist (they are read, never copied):
    make -C oracle port ld ref && python tests/golden/make_adjoint_fd.py

The case is tests/adjoint_case.py's: s=48, 11 regions, 200 cycles, the
set-up energy field plus N(0, 1e-3 e0) noise on the 1,000 elements nearest
the origin, J = sum(e * volo) over the elements whose centroid lies within
0.5 of the origin after the last cycle, 16 seeded directions.

Writes, next to this script, adjoint_fd_s48.json with
  dts, mask_idx   the time steps and the mask of the oracle's forward run of
                  the noisy field (the GPU run freezes the same ones)
  J_oracle, J_ref J of that run by the C restatement and by the reference build
  branch_fd       central differences of the oracle replaying the decision
                  tape of that run (orc_tape_replay) at relative steps 1e-6
                  to 1e-9: the derivative along the branch the run took
                  (null where a replayed run left the branch's domain: a
                  square root whose argument sits within one step of zero
                  turns negative)
  branch_fd_extended  the same replay in long double (make -C oracle ld;
                  x86 extended precision, ~2,000x less round-off), recorded on
                  its own run of the same field and steps, at relative steps
                  1e-9, 1e-10 and 1e-11
  plain_fd_ref    plain central differences of the reference build
                  (ref_step_frozen) at relative step 1e-6

The reference library runs in a child process (its error paths call exit()).
`--extended-only` recomputes branch_fd_extended into an existing fixture.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import adjoint_case as case  # noqa: E402
from oracle.oracle import OracleDomain, RefDomain  # noqa: E402

OUT = os.path.join(HERE, "adjoint_fd_s48.json")
BRANCH_STEPS = (1e-6, 1e-7, 1e-8, 1e-9)
EXTENDED_STEPS = (1e-9, 1e-10, 1e-11)
REF_STEPS = (1e-6,)


def centroid_radius(nodelist, x, y, z):
    nl = nodelist.reshape(-1, 8)
    return np.sqrt(x[nl].mean(axis=1) ** 2 + y[nl].mean(axis=1) ** 2 + z[nl].mean(axis=1) ** 2)


def finite_or_none(x):
    return float(x) if np.isfinite(x) else None


def perturbations(e, idx, rel):
    """(energy perturbations, hgcoef step) at relative step rel"""
    return case.directions(idx, e) * (rel / case.REL_STEP), rel * 3.0


def oracle_part():
    setup = OracleDomain(case.NX, case.NREG, tape=True)
    e, idx = case.initial_energy(setup.field("e").copy(), case.NX)
    setup.close()

    base = OracleDomain(case.NX, case.NREG, tape=True)
    base.field("e")[:] = e
    base.dt_record(case.NCYCLES)
    assert base.step(case.NCYCLES) == 0
    dts = base.dt_recorded(case.NCYCLES)
    mask = centroid_radius(base.field("nodelist"), base.field("x"), base.field("y"),
                           base.field("z")) < 0.5
    J0 = float(np.sum(base.field("e")[mask] * base.field("volo")[mask]))
    base.close()

    def run(e0, hg=3.0, src=None, record=False):
        d = OracleDomain(case.NX, case.NREG, hgcoef=hg, tape=True)
        d.field("e")[:] = e0
        d.dt_freeze(dts)
        if record:
            d.tape_record(case.NCYCLES)
        if src is not None:
            d.tape_replay(src)
        assert d.step(case.NCYCLES) == 0
        J = float(np.sum(d.field("e")[mask] * d.field("volo")[mask]))
        if not record:
            d.close()
            d = None
        return J, d

    Jt, rec = run(e, record=True)
    assert Jt == J0, "recording run differs from the forward run"
    Jr, _ = run(e, src=rec)
    assert Jr == J0, "replay at the recorded point differs from the forward run"
    branch = {}
    for rel in BRANCH_STEPS:
        dirs, h = perturbations(e, idx, rel)
        fd_e = [(run(e + d, src=rec)[0] - run(e - d, src=rec)[0]) / 2 for d in dirs]
        fd_h = (run(e, 3.0 + h, src=rec)[0] - run(e, 3.0 - h, src=rec)[0]) / (2 * h)
        branch[f"{rel:g}"] = {"e0": [finite_or_none(x) for x in fd_e],
                              "hgcoef": finite_or_none(fd_h)}
        print(f"branch FD at {rel:g} done", flush=True)
    return e, idx, dts, mask, J0, branch


def extended_part(e, idx, dts, mask):
    """branch-replay central differences in long double"""
    def run(e0, hg=3.0, src=None, record=False):
        d = OracleDomain(case.NX, case.NREG, hgcoef=hg, extended=True)
        d.field("e")[:] = e0
        d.dt_freeze(dts)
        if record:
            d.tape_record(case.NCYCLES)
        if src is not None:
            d.tape_replay(src)
        assert d.step(case.NCYCLES) == 0
        J = np.sum(d.field("e")[mask] * d.field("volo")[mask])
        if not record:
            d.close()
            d = None
        return J, d

    _, rec = run(e, record=True)
    ee = e.astype(np.longdouble)
    out = {}
    for rel in EXTENDED_STEPS:
        dirs, h = perturbations(e, idx, rel)
        dirs = dirs.astype(np.longdouble)
        fd_e = [(run(ee + d, src=rec)[0] - run(ee - d, src=rec)[0]) / 2 for d in dirs]
        hl = np.longdouble(h)
        fd_h = (run(ee, np.longdouble(3.0) + hl, src=rec)[0] -
                run(ee, np.longdouble(3.0) - hl, src=rec)[0]) / (2 * hl)
        out[f"{rel:g}"] = {"e0": [finite_or_none(float(x)) for x in fd_e],
                           "hgcoef": finite_or_none(float(fd_h))}
        print(f"extended branch FD at {rel:g} done", flush=True)
    return out


def ref_worker(path):
    """child process: the reference build's J and plain central differences"""
    z = np.load(path)
    e, idx, dts, mask = z["e"], z["idx"], z["dts"], z["mask"]

    def run(e0, hg=3.0):
        d = RefDomain(case.NX, case.NREG, hgcoef=hg)
        d.set_e(e0)
        d.step_frozen(dts)
        J = float(np.sum(d.field("e")[mask] * d.field("volo")[mask]))
        d.close()
        return J

    out = {"J_ref": run(e), "plain_fd_ref": {}}
    for rel in REF_STEPS:
        dirs, h = perturbations(e, idx, rel)
        out["plain_fd_ref"][f"{rel:g}"] = {
            "e0": [(run(e + d) - run(e - d)) / 2 for d in dirs],
            "hgcoef": (run(e, 3.0 + h) - run(e, 3.0 - h)) / (2 * h)}
    print(json.dumps(out))


def main():
    t0 = time.time()
    if "--extended-only" in sys.argv:
        with open(OUT) as f:
            out = json.load(f)
        setup = OracleDomain(case.NX, case.NREG)
        e, idx = case.initial_energy(setup.field("e").copy(), case.NX)
        mask = np.zeros(case.NX ** 3, bool)
        mask[out["mask_idx"]] = True
        out["branch_fd_extended"] = extended_part(e, idx, np.array(out["dts"]), mask)
        with open(OUT, "w") as f:
            json.dump(out, f, separators=(",", ":"))
        print(f"updated {OUT} in {time.time() - t0:.0f} s")
        return
    e, idx, dts, mask, J0, branch = oracle_part()
    tmp = os.path.join(HERE, "_adjoint_case.npz")
    np.savez(tmp, e=e, idx=idx, dts=dts, mask=mask)
    try:
        r = subprocess.run([sys.executable, __file__, "--ref-worker", tmp], check=True,
                           capture_output=True, text=True)
    finally:
        os.remove(tmp)
    ref = json.loads(r.stdout.strip().splitlines()[-1])
    out = {
        "case": {"nx": case.NX, "numReg": case.NREG, "ncycles": case.NCYCLES,
                 "nnoise": case.NNOISE, "ndir": case.NDIR, "radius": 0.5},
        "dts": [float(x) for x in dts],
        "mask_idx": [int(i) for i in np.flatnonzero(mask)],
        "J_oracle": J0,
        "J_ref": ref["J_ref"],
        "branch_fd": branch,
        "branch_fd_extended": extended_part(e, idx, dts, mask),
        "plain_fd_ref": ref["plain_fd_ref"],
    }
    with open(OUT, "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print(f"wrote {OUT} in {time.time() - t0:.0f} s; J oracle {J0!r} ref {ref['J_ref']!r}")


if __name__ == "__main__":
    if len(sys.argv) > 2 and sys.argv[1] == "--ref-worker":
        ref_worker(sys.argv[2])
    else:
        main()
