"""Both FP64 GPU builds against the oracle and the reference's golden fixtures.

The bar (stated by the benchmark spec): every nodal and element field within 1e-10
relative of the reference after a fixed cycle count (tests/paritylib.py
defines the elementwise relative error and its floor), the same cycle count
to stoptime with the origin energy within 1e-9 relative, and bitwise
run-to-run determinism.  Every case runs both FP64 builds: "fp64" (no
contraction, the reference's operations one by one) and "fp64-fma" (fused
multiply-add and regrouped force sums, the benchmarked build); each prints
its worst field so a log shows how far below the bar it sits.
"""
import json
import os

import numpy as np
import pytest

from paritylib import FP64_TOL, compare_states, field_rel_err

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
BUILDS = ["fp64", "fp64-fma"]


@pytest.fixture(scope="module")
def lg(native_lib):
    import lulesh_gb300
    return lulesh_gb300


def _fields():
    from lulesh_gb300 import NODE_FIELDS, ELEM_FIELDS
    return NODE_FIELDS + ELEM_FIELDS


def _check(errs, label, capsys):
    worst = max(errs, key=errs.get)
    with capsys.disabled():
        print(f"\n[parity] {label}: worst {worst} = {errs[worst]:.3e}")
    bad = {k: v for k, v in errs.items() if not v <= FP64_TOL}
    assert not bad, bad


@pytest.mark.parametrize("precision", BUILDS)
@pytest.mark.parametrize("fname", sorted(f for f in os.listdir(GOLDEN) if f.startswith("fields_")))
def test_fp64_matches_reference_golden_fields(lg, fname, precision, capsys):
    g = np.load(os.path.join(GOLDEN, fname))
    nx, nr, b, c, cyc = (int(v) for v in g["case"])
    hg, ef = (float(v) for v in g["params"])
    d = lg.Domain(nx, nr, b, c, its=cyc, hgcoef=hg, einit_factor=ef, precision=precision)
    assert d.run() == 0
    assert d.cycle == int(g["cycle"])
    _check(compare_states(d.state(), g, _fields()), f"{precision} {fname}", capsys)
    assert d.time == pytest.approx(float(g["time"]), rel=1e-12)


@pytest.fixture(scope="module")
def oracle_states(oracle_built):
    """Oracle end states, computed once per case and shared by both builds."""
    from oracle.oracle import OracleDomain
    cache = {}

    def get(nx, nr, b, c, cyc):
        key = (nx, nr, b, c, cyc)
        if key not in cache:
            o = OracleDomain(nx, nr, b, c)
            st = o.step(cyc)
            cache[key] = (st, o.state(), int(o.scalar("cycle")), o.field("e")[0])
            o.close()
        return cache[key]
    return get


@pytest.mark.parametrize("precision", BUILDS)
@pytest.mark.parametrize("case", [(30, 11, 1, 1, 100), (16, 16, 2, 4, 120), (48, 11, 1, 1, 200)])
def test_fp64_matches_oracle(lg, oracle_states, case, precision, capsys):
    nx, nr, b, c, cyc = case
    d = lg.Domain(nx, nr, b, c, its=cyc, precision=precision)
    assert d.run() == 0
    st, ref, _, _ = oracle_states(*case)
    assert st == 0
    _check(compare_states(d.state(), ref, _fields()), f"{precision} s={nx} r{nr} b{b} c{c} "
           f"{cyc} cycles", capsys)


@pytest.mark.parametrize("precision", BUILDS)
def test_fp64_to_stoptime_matches_reference_report(lg, precision):
    rep = json.load(open(os.path.join(GOLDEN, "report.json")))["s30_stoptime"]
    d = lg.Domain(30, precision=precision)
    assert d.run() == 0
    assert d.cycle == rep["cycles"] == 932
    v = d.verify()
    assert abs(v["origin_energy"] / float(rep["origin_energy"]) - 1) < 1e-6  # printed digits
    assert "%.6e" % v["origin_energy"] == rep["origin_energy"]


@pytest.mark.parametrize("precision", BUILDS)
def test_fp64_to_stoptime_matches_oracle_origin_energy(lg, oracle_states, precision, capsys):
    d = lg.Domain(30, precision=precision)
    assert d.run() == 0
    st, ref, cycles, e_ref = oracle_states(30, 11, 1, 1, 100000)
    assert st == 0
    assert d.cycle == cycles
    e_gpu = d.field("e")[0]
    rel = abs(e_gpu - e_ref) / abs(e_ref)
    with capsys.disabled():
        print(f"\n[parity] {precision} s=30 to stoptime ({cycles} cycles): origin energy "
              f"rel {rel:.3e}")
    assert rel <= 1e-9


@pytest.mark.parametrize("precision", BUILDS)
@pytest.mark.parametrize("label", ["s8_i100", "s16_r16_b2_c4_i60", "s30_i100", "s48_i200"])
def test_report_values_match_reference(lg, label, precision):
    rep = json.load(open(os.path.join(GOLDEN, "report.json")))[label]
    a = {"-s": 30, "-r": 11, "-b": 1, "-c": 1, "-i": 9999999}
    for i in range(0, len(rep["args"]), 2):
        a[rep["args"][i]] = int(rep["args"][i + 1])
    d = lg.Domain(a["-s"], a["-r"], a["-b"], a["-c"], its=a["-i"], precision=precision)
    assert d.run() == 0
    assert d.cycle == rep["cycles"]
    text = d.report(1.0)
    assert "Final Origin Energy =  %12s" % rep["origin_energy"] in text
    v = d.verify()
    assert "%.6e" % v["origin_energy"] == rep["origin_energy"]
    # the symmetry deltas are rounding-level quantities (~1e-10 absolute);
    # agreement in magnitude is the meaningful check
    for k in ("MaxAbsDiff", "TotalAbsDiff"):
        assert v[k] <= 10 * float(rep[k]) + 1e-9 * abs(v["origin_energy"]) * 1e-3


@pytest.mark.parametrize("precision", BUILDS)
def test_fp64_deterministic(lg, precision):
    st = []
    for _ in range(2):
        d = lg.Domain(20, 11, 1, 1, its=80, precision=precision)
        assert d.run() == 0
        st.append(d.state())
        d.close()
    for k in _fields():
        assert np.array_equal(st[0][k].view(np.int64), st[1][k].view(np.int64)), k


@pytest.mark.parametrize("precision", BUILDS)
def test_step_chunks_equal_one_run(lg, precision):
    a = lg.Domain(12, its=60, precision=precision)
    assert a.run() == 0
    b = lg.Domain(12, its=60, precision=precision)
    for n in (1, 7, 16, 17, 19):
        assert b.step(n) == 0
    assert b.cycle == 60
    for k in _fields():
        assert np.array_equal(a.field(k).view(np.int64), b.field(k).view(np.int64)), k


@pytest.mark.parametrize("precision", BUILDS + ["mixed"])
def test_volume_error_status(lg, precision):
    d = lg.Domain(6, 3, 1, 1, precision=precision)
    v = d.field("v")
    v[5] = -1.0
    d.set_field("v", v)
    assert d.step(1) == -1
    with pytest.raises(lg.VolumeError):
        d.step(1, check=True)


@pytest.mark.parametrize("precision", BUILDS + ["mixed"])
def test_qstop_error_status(lg, precision):
    d = lg.Domain(6, 3, 1, 1, precision=precision)
    q = d.field("q")
    q[7] = 2.0e12
    d.set_field("q", q)
    d.set_scalar("deltatime", 1.0e-16)
    assert d.step(1) == -2


@pytest.mark.parametrize("precision", BUILDS)
def test_phase_level_parity(lg, oracle_built, precision):
    from oracle.oracle import OracleDomain
    d = lg.Domain(10, 7, 1, 2, precision=precision)
    o = OracleDomain(10, 7, 1, 2)
    assert d.step(5) == 0 and o.step(5) == 0
    for ph, fields in ((0, []), (1, ["fx", "fy", "fz", "xdd", "xd", "x", "z"]),
                       (2, ["vnew", "delv", "vdov", "arealg", "ql", "qq", "e", "p", "q", "ss", "v"]),
                       (3, [])):
        assert d.phase(ph) == 0 and o.phase(ph) == 0
        sd = {f: d.field(f) for f in fields + ["vnew"]}
        so = {f: o.field(f) for f in fields + ["vnew"]}
        errs = compare_states(sd, so, fields)
        assert all(v <= FP64_TOL for v in errs.values()), (ph, errs)
    for s in ("deltatime", "time", "dtcourant", "dthydro"):
        assert d.scalar(s) == pytest.approx(o.scalar(s), rel=1e-10), s


@pytest.mark.parametrize("precision", BUILDS)
def test_large_problem_few_cycles(lg, oracle_built, precision):
    """s=150 (the benchmark mesh), 3 cycles, against the oracle."""
    from oracle.oracle import OracleDomain
    d = lg.Domain(150, its=3, precision=precision)
    assert d.run() == 0
    o = OracleDomain(150)
    o.step(3)
    for f in ("x", "xd", "e", "p", "q", "v", "ss"):
        assert field_rel_err(d.field(f), o.field(f)) <= FP64_TOL, f


@pytest.mark.parametrize("precision", BUILDS + ["mixed"])
def test_region_change_after_capture(lg, precision):
    """Replacing regNumList re-plans the material kernel's work items (their
    count, and with it the kernel variant).  A handle whose cycle graphs were
    already captured must then run exactly as one that got the new regions
    before its first cycle."""
    a = lg.Domain(12, 11, 1, 1, precision=precision)
    assert a.step(3) == 0              # captures the cycle graphs
    a.reset()
    reg = a.field("regNumList").copy()
    reg[:] = 11                        # every element in the costliest region
    reg[::7] = 1
    a.set_field("regNumList", reg)
    assert a.step(20) == 0
    b = lg.Domain(12, 11, 1, 1, precision=precision)
    b.set_field("regNumList", reg)
    assert b.step(20) == 0
    for k in _fields():
        assert np.array_equal(a.field(k).view(np.int64), b.field(k).view(np.int64)), k
