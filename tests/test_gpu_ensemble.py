"""Batched ensemble: every member must evolve exactly as the same problem run
alone through lg_create/lg_step (same arithmetic, same order), each with its
own time step and stop test, and must match the oracle run with that
member's own options (hourglass coefficient lulesh-init.cc:25, deposited
energy lulesh-init.cc:183-190, regions) within the FP64 bar."""
import numpy as np
import pytest

from paritylib import FP64_TOL, compare_states

pytestmark = pytest.mark.gpu

MEMBERS = [
    {"nx": 6, "numReg": 4, "balance": 1, "cost": 1, "its": 40, "hgcoef": 1.4, "einit_factor": 0.6},
    {"nx": 11, "numReg": 9, "balance": 1, "cost": 1, "its": 40, "hgcoef": 2.7, "einit_factor": 1.8},
    {"nx": 4, "numReg": 5, "balance": 1, "cost": 2, "its": 100, "hgcoef": 3.0, "einit_factor": 1.0},
    {"nx": 14, "numReg": 16, "balance": 2, "cost": 4, "its": 30, "hgcoef": 2.0, "einit_factor": 0.9},
    {"nx": 9, "numReg": 11, "balance": 1, "cost": 1, "its": 40, "hgcoef": 1.0, "einit_factor": 1.3},
]


def _bits(a):
    return a.view(np.int64)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_members_equal_single_problem_runs(native_lib, precision):
    import lulesh_gb300 as lg
    en = lg.Ensemble(MEMBERS, precision=precision)
    assert en.step(100) == 0
    for i, m in enumerate(MEMBERS):
        d = lg.Domain(m["nx"], m["numReg"], m["balance"], m["cost"], its=m["its"],
                      hgcoef=m["hgcoef"], einit_factor=m["einit_factor"], precision=precision)
        assert d.run() == 0
        assert en.scalar(i, "cycle") == d.cycle
        assert en.scalar(i, "time") == d.time
        for f in lg.NODE_FIELDS + lg.ELEM_FIELDS:
            assert np.array_equal(_bits(en.field(i, f)), _bits(d.field(f))), (i, f)
        d.close()
    # the s=4 member reaches stoptime (45 cycles) before its 100-cycle limit
    assert en.scalar(2, "cycle") == 45


def test_autotune_keeps_results_and_reset(native_lib):
    import lulesh_gb300 as lg
    a = lg.Ensemble(MEMBERS)
    assert a.step(20) == 0
    ref = [a.field(i, "e").copy() for i in range(len(MEMBERS))]
    b = lg.Ensemble(MEMBERS)
    choice = b.autotune(2)
    assert set(choice) == {"k_forces", "k_nodes", "k_kinematics", "k_material"}
    assert all(c["block"] in (64, 128, 256) for c in choice.values())
    assert b.scalar(0, "cycle") == 0  # the tuning cycles were undone
    assert b.step(20) == 0
    for i in range(len(MEMBERS)):
        assert np.array_equal(_bits(b.field(i, "e")), _bits(ref[i])), i


def test_sampled_ensemble_runs(native_lib):
    import lulesh_gb300 as lg
    members = lg.sample_ensemble(8, seed=0)
    for m in members:
        m["nx"] = min(m["nx"], 20)  # keep the test small
        m["its"] = 10
    en = lg.Ensemble(members)
    assert en.step(10) == 0
    assert all(en.scalar(i, "cycle") == 10 for i in range(8))


def test_members_set_up_like_single_problems(native_lib):
    """The device-built ensemble set-up: every member's fields and topology
    equal the host set-up of the same problem alone, bit for bit."""
    import lulesh_gb300 as lg
    en = lg.Ensemble(MEMBERS)
    for i, m in enumerate(MEMBERS):
        host = lg.Domain(m["nx"], m["numReg"], m["balance"], m["cost"], hgcoef=m["hgcoef"],
                         einit_factor=m["einit_factor"], device=-1)
        for f in lg.NODE_FIELDS + lg.ELEM_FIELDS:
            assert np.array_equal(_bits(en.field(i, f)), _bits(host.field(f))), (i, f)
        for f in ("nodelist", "elemBC", "regNumList"):
            assert np.array_equal(en.field(i, f), host.field(f)), (i, f)
        assert en.scalar(i, "deltatime") == host.scalar("deltatime")


def test_set_field_of_a_member(native_lib):
    """A member whose energy field is replaced evolves as the single problem
    given the same field; the other members are untouched."""
    import lulesh_gb300 as lg
    en = lg.Ensemble(MEMBERS)
    m = MEMBERS[1]
    e = en.field(1, "e")
    e[: 50] += 0.25 * e[0]
    en.set_field(1, "e", e)
    assert en.step(20) == 0
    d = lg.Domain(m["nx"], m["numReg"], m["balance"], m["cost"], its=m["its"],
                  hgcoef=m["hgcoef"], einit_factor=m["einit_factor"])
    d.set_field("e", e)
    assert d.step(20) == 0
    for f in ("e", "p", "x", "xd"):
        assert np.array_equal(_bits(en.field(1, f)), _bits(d.field(f))), f
    ref = lg.Ensemble(MEMBERS)
    assert ref.step(20) == 0
    assert np.array_equal(_bits(en.field(0, "e")), _bits(ref.field(0, "e")))
    with pytest.raises(Exception):
        en.set_field(1, "nodelist", np.zeros(8 * m["nx"] ** 3))


def test_one_member_fails_alone(native_lib):
    """Failure detection without a GPU fault: one member's first element is
    inverted on the host (a node's x moved past its neighbour), so that
    member stops with VolumeError (-1) on its first cycle; the others run on
    exactly as in an ensemble without the planted error."""
    import lulesh_gb300 as lg
    bad = 2
    en = lg.Ensemble(MEMBERS)
    x = en.field(bad, "x")
    h = x[1] - x[0]
    x[1] = x[0] - 5.0 * h          # node 1 of element 0 now left of node 0
    en.set_field(bad, "x", x)
    assert en.step(20) == -1       # the first member in error
    assert en.scalar(bad, "status") == -1
    assert en.scalar(bad, "cycle") <= 1
    clean = lg.Ensemble(MEMBERS)
    assert clean.step(20) == 0
    for i in range(len(MEMBERS)):
        if i == bad:
            continue
        assert en.scalar(i, "status") == 0
        assert en.scalar(i, "cycle") == clean.scalar(i, "cycle")
        for f in ("e", "x", "xd"):
            assert np.array_equal(_bits(en.field(i, f)), _bits(clean.field(i, f))), (i, f)


_ORACLE_MEMBERS = {}


@pytest.mark.parametrize("precision", ["fp64", "fp64-fma"])
def test_sampled_members_match_oracle(native_lib, oracle_built, precision, capsys):
    """The first 12 members of the ensemble study's seed-0 set (s in 16..64,
    hgcoef in [1, 3], energy factor in [0.5, 2], 4..16 regions), 100 cycles
    in one batched run, each against the oracle built with the member's own
    options: every field within 1e-10."""
    import lulesh_gb300 as lg
    from oracle.oracle import OracleDomain
    members = lg.sample_ensemble(12, seed=0)
    for m in members:
        m["its"] = 100
    en = lg.Ensemble(members, precision=precision)
    assert en.step(100) == 0
    fields = lg.NODE_FIELDS + lg.ELEM_FIELDS
    worst_all = 0.0
    for i, m in enumerate(members):
        key = tuple(sorted(m.items()))
        if key not in _ORACLE_MEMBERS:
            o = OracleDomain(m["nx"], m["numReg"], m["balance"], m["cost"], m["hgcoef"],
                             m["einit_factor"])
            assert o.step(100) == 0
            _ORACLE_MEMBERS[key] = o.state()
            o.close()
        ref = _ORACLE_MEMBERS[key]
        assert en.scalar(i, "cycle") == ref["cycle"] == 100
        errs = compare_states({f: en.field(i, f) for f in fields}, ref, fields)
        worst = max(errs, key=errs.get)
        worst_all = max(worst_all, errs[worst])
        with capsys.disabled():
            print(f"\n[ensemble-vs-oracle] {precision} member {i}: s={m['nx']} "
                  f"r{m['numReg']} hg {m['hgcoef']:.3f} energy x{m['einit_factor']:.3f}: "
                  f"worst {worst} = {errs[worst]:.3e}")
        assert errs[worst] <= FP64_TOL, (i, errs)
