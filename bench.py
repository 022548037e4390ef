#!/usr/bin/env python
"""bench.py -- LULESH figure of merit (element-cycles per microsecond) on GB300.

One "step" is one cycle of the reference main loop (TimeIncrement +
LagrangeLeapFrog, lulesh.cc:2745-2757) over the whole mesh.  The default
workload is the reference's built-in Sedov problem at s=150 (3,375,000
elements, 11 regions, balance 1, cost 1), 500 cycles from the initial state,
FP64 with fused multiply-add (within 1e-10 of the reference's OpenMP build on
every field after the 500 cycles; `--precision fp64` runs without
contraction).  The state (~2 GB) is larger than the 129 MB L2, so no flush is
needed between cycles.

    python bench.py [--steps 500] [--warmup 5] [--gpus N] [--impl gb300|reference]
                    [--nx 150] [--regions 11] [--balance 1] [--cost 1]
                    [--precision fp64-fma|fp64|mixed] [--ensemble N] [--err-vs-fp64]

Prints one JSON line.  `value` is the device-timed rate (CUDA events on the
handle's stream around exactly K cycles, the state resident in HBM);
`e2e` is the same metric through the C ABI with host buffers: upload of every
Domain field from pinned host memory, the K cycles, download of every field.
`subrecords` measures, in the same run, every other configuration the metric
names (config 1 at s=30; config 2's full 500 cycles in both FP64 builds; the
mixed build at s=192, 16 regions, balance 2, cost 4 with its errors against
the strict FP64 run; the 64-member ensemble batched and member by member);
`--no-subrecords` skips them.
`--impl reference` times the reference algorithm on the host cores instead
(the oracle's C restatement, -O3 OpenMP, all host threads), on the same
workload.  Under torchrun each rank runs an independent replica of the
problem on its own GPU (the path does not shard on one box); `value` sums the
element-cycles of all ranks over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "elem-cycles/µs (LULESH FOM) on 1 GB300: FP64 vs mixed/batched, err vs FP64"
UNIT = "elem-cycles/us"

# Compulsory HBM bytes per element per cycle of the persistent state each
# kernel must read or write (FP64 values, int32 indices; node quantities
# scaled by N/E).  Per-corner scratch and per-cycle temporaries are
# implementation traffic and not counted.
#   k_forces:     nodelist 32 + x,y,z,xd,yd,zd 48*N/E + p,q,v,volo,ss,elemMass 48
#   k_nodes:      read x..zd, nodalMass 56*N/E, write x..zd 48*N/E (+ the
#                 accessor fields fx..zdd 48*N/E the reference keeps)
#   k_kinematics: nodelist 32 + x..zd 48*N/E + volo, v 16 + writes vnew,
#                 delv, arealg, vdov 32
#   k_material:   lxim..lzetap 24, elemBC 4, region order 4, e,p,q,v,volo,
#                 ss,elemMass 56 read; e,p,q,v,ss 40 written
# The whole cycle's compulsory figure is 160 + 104*N/E bytes.
def alg_bytes_per_elem(kernel: str, n_over_e: float) -> float:
    return {
        "k_forces": 32 + 48 * n_over_e + 48,
        "k_nodes": (56 + 48 + 48) * n_over_e,
        "k_kinematics": 32 + 48 * n_over_e + 16 + 32,
        "k_material": 24 + 4 + 4 + 56 + 40,
    }.get(kernel, 160 + 104 * n_over_e)


# FP64 pipe lane slots per unit per launch: warp instructions issued to the
# FP64 pipe (smsp__inst_executed_pipe_fp64, every lane counted whether active
# or not, since a warp instruction holds the pipe for the same time either
# way) x 32 / units (elements; k_nodes: nodes), from ncu captures of the four
# cycle kernels of the benchmark problem (s=150, 11 regions, balance 1, cost
# 1) at cycle 10; captures of the same kernels at cycles 1 to 500 agreed to
# 0.8 %, since the elements the blast has reached stay a small share of the
# mesh.  The mixed build's counts are from s=192, 16 regions, balance 2,
# cost 4 at cycle 10.
FP64_SLOTS_PER_UNIT = {
    "fp64": {"k_forces": 1272, "k_nodes": 78.5, "k_kinematics": 699, "k_material": 391},
    "fp64-fma": {"k_forces": 648, "k_nodes": 72.5, "k_kinematics": 328, "k_material": 335},
    "mixed": {"k_forces": 24, "k_nodes": 12, "k_kinematics": 95, "k_material": 536},
}
# The workload (nx, regions, balance, cost) each build's counts were taken
# with; k_material's depend on the region mix, the others on nothing.
FP64_SLOTS_WORKLOAD = {"fp64": (150, 11, 1, 1), "fp64-fma": (150, 11, 1, 1),
                       "mixed": (192, 16, 2, 4)}
# One FP64 warp instruction per 16 cycles per SM on GB300 (ncu's
# sm__pipe_fp64_cycles_active peak): 2 lanes per SM per cycle.
FP64_LANES_PER_SM_CYCLE = 2.0


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per unit per
# launch (elements; k_nodes: nodes): the FP64 builds from the s=150
# captures above (the benchmark mesh itself, cycle 10; cycle 500 agrees to
# 0.1 %), the mixed build from s=192, 16 regions, balance 2, cost 4 (its
# benchmark mesh, cycle 10), scaled by the units a launch processes.  Well above the algorithmic bytes: the
# per-corner force scratch (k_forces writes it, k_nodes reads it) and the
# region-order gathers of k_material.
TRAFFIC_PER_UNIT = {
    "fp64": {"k_forces": 496.1, "k_nodes": 568.2, "k_kinematics": 166.4, "k_material": 291.2},
    "fp64-fma": {"k_forces": 496.1, "k_nodes": 568.1, "k_kinematics": 167.5, "k_material": 291.2},
    "mixed": {"k_forces": 219.6, "k_nodes": 277.5, "k_kinematics": 148.4, "k_material": 269.9},
}
TRAFFIC_SOURCE = {"fp64": "ncu DRAM bytes of the s=150 benchmark mesh (cycle 10)",
                  "fp64-fma": "ncu DRAM bytes of the s=150 benchmark mesh (cycle 10)",
                  "mixed": "ncu DRAM bytes per unit at s=192 r16 b2 c4 (cycle 10), scaled to the mesh"}


def _peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": d.get("hbm_gbs", 6800.0), "src": "measured"}
    return {"hbm_gbs": 6800.0, "src": "fallback"}


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict | None:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
        return dist, ws, rank, local
    return None, 1, 0, 0


def _barrier(dist):
    if dist is not None:
        dist.barrier()


def _max_over_ranks(dist, v: float) -> float:
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _workload(a) -> dict:
    return {"workload": f"Sedov blast, s={a.nx} ({a.nx ** 3} elements, {(a.nx + 1) ** 3} nodes), "
                        f"{a.regions} regions, balance {a.balance}, cost {a.cost}, "
                        f"{a.steps} cycles from the initial state, {a.precision}",
            "nx": a.nx, "regions": a.regions, "balance": a.balance, "cost": a.cost,
            "cycles": a.steps, "precision": a.precision,
            "l2": "inputs larger than L2 (resident state ~%.1f GB)" % (
                (a.nx + 1) ** 3 * 13 * 8 / 1e9 + a.nx ** 3 * (19 * 8 + 17 * 4 + 48 * 8) / 1e9),
            "parallelism": "replicas"}


def cpu_reference_rate(a, budget_s: float, warmup: int, max_cycles: int) -> dict:
    """Time the reference algorithm (oracle C restatement, OpenMP) on the host."""
    from oracle import oracle
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    t0 = time.perf_counter()
    o = oracle.OracleDomain(a.nx, a.regions, a.balance, a.cost, fast=True)
    setup = time.perf_counter() - t0
    if warmup:
        o.step(warmup)
    E = a.nx ** 3
    done, t = 0, 0.0
    while done < max_cycles and t < budget_s:
        t1 = time.perf_counter()
        st = o.step(1)
        t += time.perf_counter() - t1
        if st:
            break
        done += 1
    o.close()
    return {"value": E * done / (t * 1e6) if t > 0 else 0.0, "unit": UNIT, "cores": threads,
            "host_nproc": os.cpu_count(), "kind": "port",
            "sample": f"{done} cycles of s={a.nx} r={a.regions} b={a.balance} c={a.cost} "
                      f"after {warmup} warm-up cycles ({t:.1f} s timed, set-up {setup:.1f} s "
                      f"untimed); oracle C restatement -O3 -fopenmp, {threads} threads"}


def _total_energy(d) -> float:
    import numpy as np
    m = d.field("nodalMass")
    ke = 0.5 * np.sum(m * (d.field("xd") ** 2 + d.field("yd") ** 2 + d.field("zd") ** 2))
    return float(np.sum(d.field("e") * d.field("volo")) + ke)


def error_vs_fp64(a, d) -> dict:
    """Errors of handle d (after K cycles) against an FP64 run of the same cycles."""
    import numpy as np
    import lulesh_gb300 as lg
    d.reset()
    d.step(a.steps)
    ref = lg.Domain(a.nx, a.regions, a.balance, a.cost, its=10 ** 9, precision="fp64",
                    device=d_device(d))
    ref.step(a.steps)
    vm, vf = d.verify(), ref.verify()
    em, ef = d.field("e"), ref.field("e")
    out = {"cycles": a.steps,
           "origin_energy_rel": abs(vm["origin_energy"] / vf["origin_energy"] - 1),
           "total_energy_rel": abs(_total_energy(d) / _total_energy(ref) - 1),
           "e_normwise": float(np.max(np.abs(em - ef)) / np.max(np.abs(ef))),
           "symmetry_MaxRelDiff": vm["MaxRelDiff"], "symmetry_MaxRelDiff_fp64": vf["MaxRelDiff"],
           "symmetry_MaxAbsDiff": vm["MaxAbsDiff"], "symmetry_MaxAbsDiff_fp64": vf["MaxAbsDiff"]}
    ref.close()
    return out


def d_device(d) -> int:
    return int(os.environ.get("LOCAL_RANK", "0"))


def run_ensemble(a):
    """The batched ensemble (64 sampled Sedov problems) against the plain path run
    member by member, same members, same precision, same cycles."""
    dist, ws, rank, local = _dist()
    import numpy as np
    import lulesh_gb300 as lg
    members = lg.sample_ensemble(a.ensemble, seed=a.seed)
    for m in members:
        m["its"] = 10 ** 9
    en = lg.Ensemble(members, precision=a.precision, device=local)
    info = en.info()
    E = info["elements"]
    tune = en.autotune(3)
    if a.warmup:
        en.step(a.warmup)
    en.reset()
    l0 = en.info()["launches"]
    _barrier(dist)
    with ClockSampler(local) as clk:
        st, ms = en.step_timed(a.steps)
        _barrier(dist)
    launches = en.info()["launches"] - l0
    if st != 0:
        raise SystemExit(f"ensemble run failed with status {st}")
    ms_max = _max_over_ranks(dist, ms)
    value = ws * E * a.steps / (ms_max * 1e3)

    # end to end through the C ABI: upload every member's set-up state from
    # pinned host memory, the K cycles, download every member's fields
    fields = lg.NODE_FIELDS + lg.ELEM_FIELDS
    try:
        import torch
        pinned = torch.cuda.is_available()
    except ImportError:
        torch, pinned = None, False
    en.reset()
    host = []
    for i in range(len(members)):
        row = {}
        for f in fields:
            v = en.field(i, f)
            if pinned:
                buf = torch.empty(v.size, dtype=torch.float64, pin_memory=True).numpy()
                buf[:] = v
                v = buf
            row[f] = v
        host.append(row)
    h2d = sum(v.nbytes for row in host for v in row.values())
    _barrier(dist)
    t0 = time.perf_counter()
    for i, row in enumerate(host):
        for f, v in row.items():
            en.set_field(i, f, v)
    en.step(a.steps)
    d2h = 0
    for i in range(len(members)):
        for f in fields:
            d2h += en.field(i, f).nbytes
    t_e2e = _max_over_ranks(dist, time.perf_counter() - t0)
    e2e = {"value": ws * E * a.steps / (t_e2e * 1e6), "unit": UNIT,
           "h2d_bytes_per_step": h2d / a.steps, "d2h_bytes_per_step": d2h / a.steps}

    # the plain path, member by member (device time of each member's cycles)
    seq_ms = 0.0
    for m in members:
        d = lg.Domain(m["nx"], m["numReg"], m["balance"], m["cost"], its=10 ** 9,
                      hgcoef=m["hgcoef"], einit_factor=m["einit_factor"],
                      precision=a.precision, device=local)
        d.step(min(a.warmup, 2))
        d.reset()
        _, t = d.step_timed(a.steps)
        seq_ms += t
        d.close()
    seq_value = E * a.steps / (seq_ms * 1e3)
    sizes = [m["nx"] for m in members]
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms_max / a.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if a.precision != "mixed" else "f64+f32",
            "data": "synthetic: the reference's Sedov set-up for every member",
            "config": {"workload": f"ensemble of {len(members)} Sedov problems (seed {a.seed}): "
                                   f"s in {min(sizes)}..{max(sizes)}, {E} elements in all, "
                                   f"{a.steps} cycles, {a.precision}",
                       "members": len(members), "elements": E, "cycles": a.steps,
                       "precision": a.precision, "seed": a.seed,
                       "l2": "inputs larger than L2", "parallelism": "replicas"},
            "e2e": e2e, "gpu_launches": launches, "clocks": clk.summary(),
            "sequential_plain": {"value": seq_value, "unit": UNIT,
                                 "how": "each member alone through lg_create/lg_step_timed"},
            "batched_over_sequential": value / seq_value, "autotune": tune}
    if rank == 0 and ws == 1 and not a.no_cpu_baseline:
        line["cpu_baseline"] = cpu_ensemble_rate(members, float(
            os.environ.get("LG_CPU_BUDGET_S", "15")))
    if rank == 0:
        print(json.dumps(line), flush=True)


def cpu_ensemble_rate(members, budget_s: float) -> dict:
    """The reference algorithm (oracle port) on the members one after another."""
    from oracle import oracle
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    done_ec, t, ran = 0, 0.0, 0
    for m in members:
        if t >= budget_s:
            break
        o = oracle.OracleDomain(m["nx"], m["numReg"], m["balance"], m["cost"], m["hgcoef"],
                                m["einit_factor"], fast=True)
        c = 0
        while c < 300 and t < budget_s:
            t1 = time.perf_counter()
            o.step(1)
            t += time.perf_counter() - t1
            c += 1
        done_ec += c * m["nx"] ** 3
        ran += 1
        o.close()
    return {"value": done_ec / (t * 1e6) if t else 0.0, "unit": UNIT, "cores": threads,
            "host_nproc": os.cpu_count(), "kind": "port",
            "sample": f"the first {ran} members in order, up to 300 cycles each, "
                      f"{t:.1f} s timed; oracle C restatement, {threads} threads"}


def run_reference(a):
    dist, ws, rank, local = _dist()
    if rank != 0:
        return
    base = cpu_reference_rate(a, budget_s=float(os.environ.get("LG_REF_BUDGET_S", "120")),
                              warmup=min(a.warmup, 2), max_cycles=a.steps)
    line = {"metric": METRIC, "value": base["value"], "unit": UNIT, "n_gpus": ws,
            "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": (a.nx ** 3 / base["value"] / 1e3) if base["value"] else None,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: the reference's built-in Sedov problem set-up",
            "config": _workload(a), "impl": "reference", "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _timed_single(lg, nx, nr, b, c, cycles, precision, device, warmup=3):
    """A fresh problem: warm-up cycles, reset, then `cycles` device-timed
    cycles from the initial state.  Returns (handle, record)."""
    d = lg.Domain(nx, nr, b, c, its=10 ** 9, precision=precision, device=device)
    if warmup:
        d.step(warmup)
    d.reset()
    st, ms = d.step_timed(cycles)
    if st != 0:
        raise SystemExit(f"s={nx} {precision}: run failed with status {st}")
    return d, {"value": nx ** 3 * cycles / (ms * 1e3), "unit": UNIT, "cycles": cycles,
               "ms_per_cycle": ms / cycles, "precision": precision,
               "origin_energy": d.field("e")[0]}


def _errors(d, ref) -> dict:
    """Errors of handle d against handle ref after the same cycles: origin
    energy, total energy (internal + kinetic), the energy field normwise, and
    both runs' plane-0 symmetry deltas (lulesh-util.cc:197-212)."""
    import numpy as np
    vm, vf = d.verify(), ref.verify()
    em, ef = d.field("e"), ref.field("e")
    return {"origin_energy_rel": abs(vm["origin_energy"] / vf["origin_energy"] - 1),
            "total_energy_rel": abs(_total_energy(d) / _total_energy(ref) - 1),
            "e_normwise": float(np.max(np.abs(em - ef)) / np.max(np.abs(ef))),
            "symmetry_MaxRelDiff": vm["MaxRelDiff"], "symmetry_MaxRelDiff_ref": vf["MaxRelDiff"],
            "symmetry_MaxAbsDiff": vm["MaxAbsDiff"], "symmetry_MaxAbsDiff_ref": vf["MaxAbsDiff"]}


def _ensemble_rates(lg, members, precision, cycles, device, warmup=2) -> dict:
    """Batched rate of the members (autotuned, device-timed) and the plain
    path's rate running them one by one, same cycles."""
    en = lg.Ensemble(members, precision=precision, device=device)
    E = en.info()["elements"]
    tune = en.autotune(3)
    if warmup:
        en.step(warmup)
    en.reset()
    st, ms = en.step_timed(cycles)
    if st != 0:
        raise SystemExit(f"ensemble {precision}: status {st}")
    en.close()
    seq_ms = 0.0
    for m in members:
        d = lg.Domain(m["nx"], m["numReg"], m["balance"], m["cost"], its=10 ** 9,
                      hgcoef=m["hgcoef"], einit_factor=m["einit_factor"],
                      precision=precision, device=device)
        d.step(warmup)
        d.reset()
        _, t = d.step_timed(cycles)
        seq_ms += t
        d.close()
    batched, seq = E * cycles / (ms * 1e3), E * cycles / (seq_ms * 1e3)
    return {"value": batched, "unit": UNIT, "sequential_plain": seq,
            "batched_over_sequential": batched / seq, "elements": E, "cycles": cycles,
            "precision": precision, "autotune": {k: v["block"] * (-1 if v["persistent"] else 1)
                                                  for k, v in tune.items()}}


def subrecords(a, device: int) -> dict:
    """Every configuration the metric names, measured in the same run as the
    headline (device-timed, each from its initial state after warm-up):
      config1:      s=30, 11 regions, 100 cycles, each arithmetic
      config2_full: s=150, 11 regions, 500 cycles, both FP64 builds
      mixed:        s=192, 16 regions, balance 2, cost 4, 500 cycles: mixed and
                    strict FP64 (the error reference), FP64+FMA over 100 cycles
      ensemble:     the 64-member study set (seed 0), 300 cycles, batched and
                    member by member, FP64+FMA and mixed"""
    import lulesh_gb300 as lg
    out = {}
    c1 = {}
    for prec in ("fp64", "fp64-fma", "mixed"):
        d, r = _timed_single(lg, 30, 11, 1, 1, 100, prec, device)
        c1[prec] = r
        d.close()
    out["config1"] = {"workload": "Sedov s=30 (27,000 elements), 11 regions, b1 c1, 100 cycles",
                      **c1}
    c2 = {}
    for prec in ("fp64-fma", "fp64"):
        d, r = _timed_single(lg, 150, 11, 1, 1, 500, prec, device)
        c2[prec] = r
        d.close()
    out["config2_full"] = {"workload": "Sedov s=150 (3,375,000 elements), 11 regions, b1 c1, "
                                       "500 cycles", **c2}
    dm, rm = _timed_single(lg, 192, 16, 2, 4, 500, "mixed", device)
    df, rf = _timed_single(lg, 192, 16, 2, 4, 500, "fp64", device)
    err = _errors(dm, df)
    dm.close()
    df.close()
    dfa, rfa = _timed_single(lg, 192, 16, 2, 4, 100, "fp64-fma", device)
    dfa.close()
    out["mixed"] = {"workload": "Sedov s=192 (7,077,888 elements), 16 regions, balance 2, cost "
                                "4, 500 cycles", "mixed": rm, "fp64": rf, "fp64-fma_100_cycles": rfa,
                    "mixed_over_fp64": rm["value"] / rf["value"],
                    "mixed_over_fp64_fma": rm["value"] / rfa["value"],
                    "err_vs_fp64": err,
                    "err_reference": "the strict FP64 GPU run of the same 500 cycles"}
    members = lg.sample_ensemble(64, seed=0)
    for m in members:
        m["its"] = 10 ** 9
    out["ensemble"] = {"workload": "64 sampled Sedov problems (seed 0: s 16..64, energy x "
                                   "[0.5, 2], hgcoef [1, 3], 4..16 regions), 300 cycles",
                       "fp64-fma": _ensemble_rates(lg, members, "fp64-fma", 300, device),
                       "mixed": _ensemble_rates(lg, members, "mixed", 300, device)}
    return out


def run_gpu(a):
    dist, ws, rank, local = _dist()
    import numpy as np
    import lulesh_gb300 as lg
    try:
        import torch
        sync = torch.cuda.synchronize if torch.cuda.is_available() else (lambda: None)
    except ImportError:
        torch, sync = None, (lambda: None)

    E, N = a.nx ** 3, (a.nx + 1) ** 3
    d = lg.Domain(a.nx, a.regions, a.balance, a.cost, its=10 ** 9, precision=a.precision,
                  device=local)
    # warm-up cycles, then back to the initial state
    if a.warmup:
        d.step(a.warmup)
    d.reset()

    # device-timed region: exactly K cycles
    launches0 = d.scalar("launches")
    _barrier(dist)
    sync()
    with ClockSampler(local) as clk:
        st, ms = d.step_timed(a.steps)
        sync()
        _barrier(dist)
    launches = int(d.scalar("launches") - launches0)
    if st != 0:
        raise SystemExit(f"run failed with status {st}")
    ms_max = _max_over_ranks(dist, ms)
    value = ws * E * a.steps / (ms_max * 1e3)
    verify = d.verify()

    # per-kernel device times over a profiled pass of the same cycles
    d.reset()
    prof_cycles = min(a.steps, 20)
    prof = d.profile(prof_cycles)
    total = sum(prof.values())
    dom = max(prof, key=prof.get)
    avg_ms = prof[dom] / prof_cycles
    peaks = _peaks()
    ab = alg_bytes_per_elem(dom, N / E) * E
    achieved = ab / (avg_ms * 1e-3) / 1e9
    per_unit = TRAFFIC_PER_UNIT.get(a.precision, {}).get(dom)
    traffic = None if per_unit is None else per_unit * (N if dom == "k_nodes" else E)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"], "traffic": traffic,
                "traffic_source": TRAFFIC_SOURCE.get(a.precision) if traffic else None,
                "kernel": dom,
                "peak_source": peaks["src"], "alg_bytes_per_launch": ab,
                "kernel_ms_per_launch": avg_ms,
                "kernel_share": {k: v / total for k, v in prof.items()}}
    # FP64 pipe roofline (the bound of this path)
    # FP64 pipe roofline (the bound of this path): the dominant kernel's pipe
    # lane slots per launch over its time, against the pipe's issue rate at
    # the SM clock sampled during the timed region; the DFMA
    # microbenchmark's rate is reported beside it
    import torch
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    clk_sum = clk.summary() or {}
    sm_hz = (clk_sum.get("sm_mhz") or 2070.0) * 1e6
    pipe_peak = FP64_LANES_PER_SM_CYCLE * sms * sm_hz / 1e9
    slots = FP64_SLOTS_PER_UNIT.get(a.precision, {})
    roof64 = {"bound": "fp64_pipe", "unit": "G FP64 lane-inst/s", "kernel": dom,
              "peak": pipe_peak, "peak_source": f"2 lanes/SM/cycle x {sms} SMs x "
                                                f"{sm_hz / 1e6:.0f} MHz (sampled)",
              "dfma_microbenchmark": lg.measure_pipe("fma")}
    if FP64_SLOTS_WORKLOAD.get(a.precision) == (a.nx, a.regions, a.balance, a.cost) and slots:
        per_unit = slots.get(dom)
        units = N if dom == "k_nodes" else E
        ach = per_unit * units / (avg_ms * 1e-3) / 1e9
        cyc_slots = sum(slots[k] * (N / E if k == "k_nodes" else 1.0) for k in slots)
        cyc_ach = cyc_slots * E * a.steps / (ms_max * 1e-3) / 1e9
        roof64.update({"achieved": ach, "frac": ach / pipe_peak, "slots_per_unit": per_unit,
                       "cycle_slots_per_elem": cyc_slots, "cycle_achieved": cyc_ach,
                       "cycle_frac": cyc_ach / pipe_peak})

    # end to end through the C ABI with host buffers
    fields = lg.NODE_FIELDS + lg.ELEM_FIELDS
    if torch is not None and torch.cuda.is_available():
        host = {f: torch.empty(d.field_info(f)[0], dtype=torch.float64,
                               pin_memory=True).numpy() for f in fields}
    else:
        host = {f: np.empty(d.field_info(f)[0]) for f in fields}
    d.reset()
    for f in fields:
        d.field(f, out=host[f])
    init = {f: host[f].copy() for f in fields}
    h2d = sum(host[f].nbytes for f in fields)
    # the median of several end-to-end runs, each from the initial state: on
    # a shared host some uploads or downloads of the 709 MB took 25-90 ms
    # instead of 4 (phase_seconds shows which), a stall not seen on a fresh
    # host
    reps = 5 if a.steps <= 100 else 3
    times, st2 = [], 0
    phases = {"h2d": [], "cycles": [], "d2h": []}  # host clock, per run
    for _ in range(reps):
        d.reset()  # the time-step state back to cycle 0 (untimed)
        for f in fields:
            host[f][:] = init[f]
        _barrier(dist)
        t0 = time.perf_counter()
        for f in fields:
            d.set_field(f, host[f])
        t1 = time.perf_counter()
        st2 = d.step(a.steps) or st2
        t2 = time.perf_counter()
        for f in fields:
            d.field(f, out=host[f])
        t3 = time.perf_counter()
        times.append(t3 - t0)
        for k, v in zip(phases, (t1 - t0, t2 - t1, t3 - t2)):
            phases[k].append(round(v, 5))
        _barrier(dist)
    t_e2e = _max_over_ranks(dist, statistics.median(times))
    e2e = {"value": ws * E * a.steps / (t_e2e * 1e6), "unit": UNIT,
           "h2d_bytes_per_step": h2d / a.steps, "d2h_bytes_per_step": h2d / a.steps,
           "status": st2, "runs": reps, "run_seconds": times, "phase_seconds": phases}

    # the same when the caller keeps the reference's Domain on the host and
    # syncs it around every cycle (the second binding of the integration
    # guide): every field up, one cycle, every field down, a few cycles
    nsync = min(a.steps, 10)
    d.reset()
    _barrier(dist)
    t0 = time.perf_counter()
    for _ in range(nsync):
        for f in fields:
            d.set_field(f, host[f])
        d.step(1)
        for f in fields:
            d.field(f, out=host[f])
    t_sync = _max_over_ranks(dist, time.perf_counter() - t0)
    e2e_host = {"value": ws * E * nsync / (t_sync * 1e6), "unit": UNIT, "cycles": nsync,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": h2d,
                "how": "every Domain field from pinned host memory, lg_step(1), every field "
                       "back, per cycle"}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms_max / a.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if a.precision != "mixed" else "f64+f32",
            "data": "synthetic: the reference's built-in Sedov problem set-up",
            "config": _workload(a), "e2e": e2e, "e2e_host_domain": e2e_host,
            "gpu_launches": launches, "roofline": roofline, "roofline_fp64": roof64, "clocks": clk.summary(),
            "origin_energy": verify["origin_energy"]}
    if a.err_vs_fp64 and a.precision != "fp64":
        line["err_vs_fp64"] = error_vs_fp64(a, d)
    d.close()
    if ws == 1 and not a.no_subrecords:
        with ClockSampler(local) as clk_sub:
            t_sub = time.perf_counter()
            line["subrecords"] = subrecords(a, local)
            line["subrecords"]["wall_s"] = time.perf_counter() - t_sub
        line["subrecords"]["clocks"] = clk_sub.summary()
    if rank == 0 and ws == 1 and not a.no_cpu_baseline:
        line["cpu_baseline"] = cpu_reference_rate(
            a, budget_s=float(os.environ.get("LG_CPU_BUDGET_S", "15")), warmup=1,
            max_cycles=a.steps)
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    p = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=None,
                   help="cycles to time (default 500; 300 with --ensemble)")
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    p.add_argument("--nx", type=int, default=150)
    p.add_argument("--regions", type=int, default=11)
    p.add_argument("--balance", type=int, default=1)
    p.add_argument("--cost", type=int, default=1)
    p.add_argument("--precision", default="fp64-fma", choices=["fp64", "fp64-fma", "mixed"],
                   help="fp64-fma (default): FP64 with fused multiply-add, within 1e-10 of "
                        "the reference at s=150/500 cycles; fp64: no contraction (the "
                        "reference's arithmetic operation for operation); mixed: FP32 "
                        "forces/kinematics/Q with FP64 state and EOS")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-subrecords", action="store_true",
                   help="skip the other configurations' records (config 1, config 2 over 500 "
                        "cycles, mixed s=192, the 64-member ensemble; about 80 s)")
    p.add_argument("--ensemble", type=int, default=0,
                   help="batched ensemble of this many sampled problems instead of one problem")
    p.add_argument("--seed", type=int, default=0, help="ensemble sample seed")
    p.add_argument("--err-vs-fp64", action="store_true",
                   help="after timing, rerun the workload in FP64 (untimed) and report the "
                        "origin-energy, total-energy and field errors of this precision")
    a = p.parse_args()
    if a.steps is None:
        a.steps = 300 if a.ensemble else 500
    if a.warmup < 0 or a.steps < 1:
        p.error("need --steps >= 1 and --warmup >= 0")
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    if a.impl == "reference":
        run_reference(a)
    elif a.ensemble:
        run_ensemble(a)
    else:
        run_gpu(a)


if __name__ == "__main__":
    main()
