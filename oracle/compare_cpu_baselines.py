"""Time the reference's own CPU build next to the oracle port (test
infrastructure: it measures the CPU baselines, it is not part of the product).

    make -C oracle port stock && python oracle/compare_cpu_baselines.py [--threads N]

For each case it runs, best of 3 each:
  * the reference CLI built with its own Makefile's flags (-O3 -fopenmp;
    oracle/_ref/lulesh_ref_stock), taking elem-cycles/us = 1 / grind from the
    reference's own report line (lulesh-util.cc:185-227); the grind time
    covers the cycle loop only (lulesh.cc:2736-2767);
  * the oracle restatement's default-contraction build
    (oracle/build/liblulesh_oracle_fast.so, -O3 -fopenmp), which bench.py's
    reference arm times on hosts without the reference sources, over the same
    cycles from the same initial state, set-up excluded.
Prints one JSON line per case and a summary line with the host's nproc and
the threads used.  Where the reference build is missing it says so and exits 0.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import re
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
# run as a script, this directory comes first on sys.path and its oracle.py
# would shadow the oracle package
sys.path[:] = [ROOT] + [p for p in sys.path if os.path.abspath(p or ".") != HERE]
STOCK = os.path.join(HERE, "_ref", "lulesh_ref_stock")

CASES = [(30, 11, 1, 1, 100), (60, 11, 1, 1, 40), (150, 11, 1, 1, 8)]


def reference_rate(nx, nr, b, c, its, threads) -> float:
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    out = subprocess.run([STOCK, "-s", str(nx), "-r", str(nr), "-b", str(b), "-c", str(c),
                          "-i", str(its)], capture_output=True, text=True, env=env,
                         check=True).stdout
    grind = float(re.search(r"Grind time \(us/z/c\)\s*=\s*([0-9.eE+-]+)", out).group(1))
    return 1.0 / grind


def port_rate(nx, nr, b, c, its) -> float:
    from oracle.oracle import OracleDomain
    o = OracleDomain(nx, nr, b, c, fast=True)
    t0 = time.perf_counter()
    st = o.step(its)
    t = time.perf_counter() - t0
    o.close()
    if st:
        raise RuntimeError(f"port run failed: {st}")
    return nx ** 3 * its / (t * 1e6)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count())
    ap.add_argument("--repeats", type=int, default=3)
    a = ap.parse_args()
    if not os.path.exists(STOCK):
        print(json.dumps({"unavailable": "reference build oracle/_ref/lulesh_ref_stock missing "
                                         "(its sources are not on this host)"}))
        return
    os.environ["OMP_NUM_THREADS"] = str(a.threads)
    rows = []
    for case in CASES:
        ref = max(reference_rate(*case, a.threads) for _ in range(a.repeats))
        port = max(port_rate(*case) for _ in range(a.repeats))
        row = {"s": case[0], "regions": case[1], "balance": case[2], "cost": case[3],
               "cycles": case[4], "reference_elem_cycles_per_us": ref,
               "port_elem_cycles_per_us": port, "port_over_reference": port / ref}
        rows.append(row)
        print(json.dumps(row), flush=True)
    print(json.dumps({"host": platform.machine(), "nproc": os.cpu_count(),
                      "threads": a.threads, "best_of": a.repeats,
                      "cpu": platform.processor() or None}))


if __name__ == "__main__":
    main()
