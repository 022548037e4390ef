"""The parity bar sees small changes of the model.

The GPU parity tests hold every field within FP64_TOL (1e-10) of the oracle,
by the metric of tests/paritylib.py.  Here the oracle runs the same small
problem twice, the second time with a planted change of 1e-9 (relative) in
one problem parameter, and that metric must put the two runs beyond
FP64_TOL: a kernel whose arithmetic moved its results that far would fail
the GPU tests.  An unchanged second run must compare as zero.

Problem: s=10, 5 regions, balance 1, cost 2, hgcoef 1.6, energy x0.7, 60
cycles (the golden fixture fields_s10_r5_b1_c2_i60_hg1.6_ef0.7).
"""
import pytest

from paritylib import FP64_TOL, compare_states

CASE = dict(nx=10, numReg=5, balance=1, cost=2)
HG, EF, CYCLES = 1.6, 0.7, 60


def _run(hg: float, ef: float) -> dict:
    from oracle.oracle import OracleDomain
    d = OracleDomain(CASE["nx"], CASE["numReg"], CASE["balance"], CASE["cost"], hg, ef)
    assert d.step(CYCLES) == 0
    out = d.state()
    d.close()
    return out


def _worst(a: dict, b: dict) -> float:
    from oracle.oracle import ELEM_FIELDS, NODE_FIELDS
    errs = compare_states(a, b, NODE_FIELDS + ELEM_FIELDS)
    return max(errs.values())


def test_unchanged_rerun_compares_as_zero(oracle_built):
    assert _worst(_run(HG, EF), _run(HG, EF)) == 0.0


@pytest.mark.parametrize("which", ["hgcoef", "energy"])
def test_planted_change_exceeds_the_bar(oracle_built, which):
    ref = _run(HG, EF)
    planted = _run(HG * (1 + 1e-9), EF) if which == "hgcoef" else _run(HG, EF * (1 + 1e-9))
    worst = _worst(planted, ref)
    print(f"[sensitivity] {which} x (1 + 1e-9): worst field {worst:.3e} (bar {FP64_TOL:.0e})")
    assert worst > FP64_TOL
