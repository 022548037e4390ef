"""How far the reference moves from itself when compiled with FMA contraction
(test infrastructure: it measures the reference, it is not part of the product).

    make -C oracle port ref ref-fma && python oracle/fma_spread.py [--nx 150] [--cycles 500]

Runs the unchanged reference sources twice over the same problem: the
uncontracted build (_ref/liblulesh_ref.so, -ffp-contract=off, the parity
oracle's arithmetic) and the contracted one (_ref/liblulesh_ref_fma.so,
-ffp-contract=fast with FMA instructions, what gcc does by default on an FMA
host such as the GPU machine's Grace cores).  Prints one JSON line: the worst
elementwise relative difference per field, with the parity tests' metric
(tests/paritylib.py: |a_i - b_i| / max(|b_i|, 1e-6 max_j |b_j|)).
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
# run as a script, this directory comes first on sys.path and its oracle.py
# would shadow the oracle package
sys.path[:] = [ROOT, os.path.join(ROOT, "tests")] + \
    [p for p in sys.path if os.path.abspath(p or ".") != HERE]

from oracle.oracle import ELEM_FIELDS, NODE_FIELDS, REF_LIB, RefDomain  # noqa: E402
from paritylib import compare_states  # noqa: E402

FMA_LIB = os.path.join(HERE, "_ref", "liblulesh_ref_fma.so")


def run(lib: str, nx: int, cycles: int) -> tuple[dict, float]:
    d = RefDomain(nx, lib_path=lib)
    t0 = time.perf_counter()
    done = d.step(cycles)  # the reference's cycle count afterwards
    dt = time.perf_counter() - t0
    if done != cycles:
        raise RuntimeError(f"{lib}: stopped at cycle {done}")
    out = d.state()
    d.close()
    return out, dt


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--nx", type=int, default=150)
    ap.add_argument("--cycles", type=int, default=500)
    a = ap.parse_args()
    for lib in (REF_LIB, FMA_LIB):
        if not os.path.exists(lib):
            print(json.dumps({"unavailable": f"{os.path.basename(lib)} not built"}))
            return 0
    strict, t_strict = run(REF_LIB, a.nx, a.cycles)
    fma, t_fma = run(FMA_LIB, a.nx, a.cycles)
    fields = NODE_FIELDS + ELEM_FIELDS
    errs = compare_states(fma, strict, fields)
    worst = max(errs, key=errs.get)
    print(json.dumps({"nx": a.nx, "cycles": a.cycles, "worst_field": worst,
                      "worst": errs[worst], "per_field": {k: float(f"{v:.2e}") for k, v in errs.items()},
                      "origin_energy": [strict["e"][0], fma["e"][0]],
                      "seconds": [round(t_strict, 1), round(t_fma, 1)],
                      "host": os.uname().machine, "threads": os.cpu_count()}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
