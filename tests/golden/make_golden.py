"""Generate the golden fixtures from the UNCHANGED reference build.

Run where the reference sources exist (they are read, never copied):
    make -C oracle ref && python tests/golden/make_golden.py

Writes, next to this script:
  report.json   end-of-run report values of the reference CLI (oracle/_ref/lulesh_ref)
                for several option sets, parsed from its own output
  setup.json    SHA-256 digests of the reference Domain's set-up arrays
                (regNumList, nodelist, elemBC, nodalMass, volo) for several sizes
  fields_*.npz  every nodal and element field of the reference Domain after a
                fixed number of cycles, for small problems

The reference library is driven in a child process per case because its
error paths call exit().
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

REPORT_CASES = [
    # (args, label)
    (["-s", "8", "-i", "100"], "s8_i100"),
    (["-s", "16", "-r", "16", "-b", "2", "-c", "4", "-i", "60"], "s16_r16_b2_c4_i60"),
    (["-s", "30", "-i", "100"], "s30_i100"),
    (["-s", "30"], "s30_stoptime"),
    (["-s", "48", "-i", "200"], "s48_i200"),
]

FIELD_CASES = [
    # (nx, numReg, balance, cost, cycles, hgcoef, einit_factor)
    (8, 11, 1, 1, 50, 3.0, 1.0),
    (12, 16, 2, 4, 40, 3.0, 1.0),
    (10, 5, 1, 2, 60, 1.6, 0.7),
]

SETUP_CASES = [(30, 11, 1, 1), (48, 11, 1, 1), (16, 16, 2, 4), (20, 4, 3, 1), (7, 1, 1, 1)]


def parse_report(text: str) -> dict:
    def grab(key):
        m = re.search(re.escape(key) + r"\s*=\s*([-+0-9.eE]+)", text)
        return m.group(1) if m else None
    return {
        "cycles": int(grab("Iteration count")),
        "origin_energy": grab("Final Origin Energy"),
        "MaxAbsDiff": grab("MaxAbsDiff"),
        "TotalAbsDiff": grab("TotalAbsDiff"),
        "MaxRelDiff": grab("MaxRelDiff"),
    }


def _digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def child_fields(case, out):
    from oracle.oracle import RefDomain, NODE_FIELDS, ELEM_FIELDS, SCALARS
    nx, nr, b, c, cyc, hg, ef = case
    r = RefDomain(nx, nr, b, c, hg, ef)
    r.step(cyc)
    st = r.state()
    np.savez_compressed(out, **{k: np.asarray(v) for k, v in st.items()},
                        case=np.array([nx, nr, b, c, cyc], dtype=np.int64),
                        params=np.array([hg, ef]))


def child_setup(case) -> dict:
    from oracle.oracle import RefDomain
    nx, nr, b, c = case
    r = RefDomain(nx, nr, b, c)
    out = {k: _digest(r.field(k)) for k in ("regNumList", "nodelist", "elemBC", "nodalMass",
                                               "volo")}
    out["deltatime"] = float(r.scalar("deltatime")).hex()
    return out


def main():
    from oracle import oracle
    oracle.build(ref=True)
    env = dict(os.environ, OMP_NUM_THREADS=os.environ.get("OMP_NUM_THREADS", "4"))
    reports = {}
    for args, label in REPORT_CASES:
        txt = subprocess.run([oracle.REF_BIN] + args, capture_output=True, text=True, env=env,
                             check=True).stdout
        reports[label] = {"args": args, **parse_report(txt)}
        print(label, reports[label])
    with open(os.path.join(HERE, "report.json"), "w") as f:
        json.dump(reports, f, indent=1)

    setup = {}
    for case in SETUP_CASES:
        code = ("import sys, json; sys.path.insert(0, %r); sys.path.insert(0, %r); "
                "import make_golden as g; print(json.dumps(g.child_setup(%r)))"
                % (ROOT, HERE, case))
        res = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True,
                             env=env, check=True)
        setup["_".join(map(str, case))] = json.loads(res.stdout.strip().splitlines()[-1])
    with open(os.path.join(HERE, "setup.json"), "w") as f:
        json.dump(setup, f, indent=1)

    for case in FIELD_CASES:
        name = "fields_s%d_r%d_b%d_c%d_i%d_hg%g_ef%g.npz" % case
        out = os.path.join(HERE, name)
        code = ("import sys; sys.path.insert(0, %r); sys.path.insert(0, %r); "
                "import make_golden as g; g.child_fields(%r, %r)" % (ROOT, HERE, case, out))
        subprocess.run([sys.executable, "-c", code], env=env, check=True)
        print("wrote", name, os.path.getsize(out))


if __name__ == "__main__":
    main()
