"""The oracle restatement, pinned against the reference.

The golden fixtures in tests/golden/ were produced by the unchanged reference
sources (tests/golden/make_golden.py).  Where the reference build exists on
this host, the restatement is also compared with it directly.
"""
import hashlib
import json
import os
import subprocess
import sys

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _bits(a):
    return np.ascontiguousarray(a).view(np.int64 if a.dtype == np.float64 else np.int32)


def _field_cases():
    return sorted(f for f in os.listdir(GOLDEN) if f.startswith("fields_"))


@pytest.mark.parametrize("fname", _field_cases())
def test_oracle_fields_match_reference_golden(oracle_built, fname):
    from oracle.oracle import OracleDomain, NODE_FIELDS, ELEM_FIELDS
    g = np.load(os.path.join(GOLDEN, fname))
    nx, nr, b, c, cyc = (int(v) for v in g["case"])
    hg, ef = (float(v) for v in g["params"])
    o = OracleDomain(nx, nr, b, c, hg, ef)
    assert o.step(cyc) == 0
    for k in NODE_FIELDS + ELEM_FIELDS:
        assert np.array_equal(_bits(o.field(k)), _bits(g[k])), k
    for s in ("time", "deltatime", "dtcourant", "dthydro", "cycle"):
        assert o.scalar(s) == float(g[s]), s


def _report_values(o, nx):
    e = o.field("e")
    mx = tot = mr = 0.0
    for j in range(nx):
        for k in range(j + 1, nx):
            ad = abs(e[j * nx + k] - e[k * nx + j])
            tot += ad
            mx = max(mx, ad)
            with np.errstate(divide="ignore", invalid="ignore"):
                rd = ad / e[k * nx + j]
            mr = max(mr, rd)
    return e[0], mx, tot, mr


def _args_to_case(args):
    d = {"-s": 30, "-r": 11, "-b": 1, "-c": 1, "-i": 9999999}
    for i in range(0, len(args), 2):
        d[args[i]] = int(args[i + 1])
    return d


@pytest.mark.parametrize("label", ["s8_i100", "s16_r16_b2_c4_i60", "s30_i100"])
def test_oracle_report_matches_reference_golden(oracle_built, label):
    from oracle.oracle import OracleDomain
    rep = json.load(open(os.path.join(GOLDEN, "report.json")))[label]
    a = _args_to_case(rep["args"])
    o = OracleDomain(a["-s"], a["-r"], a["-b"], a["-c"])
    o.step(a["-i"])
    assert int(o.scalar("cycle")) == rep["cycles"]
    e0, mx, tot, mr = _report_values(o, a["-s"])
    assert "%.6e" % e0 == rep["origin_energy"]
    assert "%.6e" % mx == rep["MaxAbsDiff"]
    assert "%.6e" % tot == rep["TotalAbsDiff"]
    assert "%.6e" % mr == rep["MaxRelDiff"]


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("key", list(json.load(open(os.path.join(GOLDEN, "setup.json")))))
def test_oracle_setup_matches_reference_golden(oracle_built, key):
    from oracle.oracle import OracleDomain
    want = json.load(open(os.path.join(GOLDEN, "setup.json")))[key]
    nx, nr, b, c = (int(v) for v in key.split("_"))
    o = OracleDomain(nx, nr, b, c)
    for f in ("regNumList", "nodelist", "elemBC", "nodalMass", "volo"):
        assert _digest(o.field(f)) == want[f], f
    assert float(o.scalar("deltatime")).hex() == want["deltatime"]


def test_oracle_thread_count_invariant(oracle_built):
    """The corner-gather semantics make the result independent of threads."""
    code = ("import sys; sys.path.insert(0, %r); from oracle.oracle import OracleDomain; "
            "import hashlib; o = OracleDomain(10, 7, 1, 2); o.step(40); "
            "print(hashlib.sha256(b''.join(o.field(f).tobytes() for f in "
            "['x','xd','e','p','q','v','ss'])).hexdigest())"
            % os.path.dirname(GOLDEN.rstrip("/")).rsplit("/tests", 1)[0])
    outs = set()
    for t in ("1", "3"):
        env = dict(os.environ, OMP_NUM_THREADS=t)
        r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True,
                           env=env, check=True)
        outs.add(r.stdout.strip())
    assert len(outs) == 1


def test_oracle_error_status_volume(oracle_built):
    """A collapsed element makes the step return VolumeError (-1), not exit."""
    from oracle.oracle import OracleDomain
    o = OracleDomain(6, 3, 1, 1)
    o.field("v")[5] = -1.0
    assert o.step(1) == -1


def test_oracle_error_status_qstop(oracle_built):
    from oracle.oracle import OracleDomain
    o = OracleDomain(6, 3, 1, 1)
    o.field("q")[7] = 2.0e12
    # a tiny first step keeps the large stress from collapsing the element
    # before the qstop test (lulesh.cc:1993-2008) is reached
    o.set_scalar("deltatime", 1.0e-16)
    assert o.step(1) == -2


def test_restatement_matches_reference_directly(oracle_built):
    """Bit-for-bit against the unchanged reference build (when present here)."""
    from oracle import oracle
    if not oracle.ref_available():
        pytest.skip("reference build not present on this host")
    code = """
import sys; sys.path.insert(0, %r)
import numpy as np
from oracle.oracle import OracleDomain, RefDomain, NODE_FIELDS, ELEM_FIELDS
for case in [(9, 11, 1, 1, 70, 3.0, 1.0), (11, 16, 2, 4, 50, 2.2, 1.4)]:
    o = OracleDomain(*case[:4], case[5], case[6]); r = RefDomain(*case[:4], case[5], case[6])
    o.step(case[4]); r.step(case[4])
    for k in NODE_FIELDS + ELEM_FIELDS:
        assert np.array_equal(o.field(k).view(np.int64), r.field(k).view(np.int64)), k
print("ok")
""" % os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True,
                       env=dict(os.environ, OMP_NUM_THREADS="4"))
    assert r.returncode == 0 and "ok" in r.stdout, r.stderr


def _noisy_case(lib_kw, nx=10, ncyc=30):
    """the adjoint study's kind of input on a small mesh: the set-up field
    with N(0, 1e-3 e0) noise near the origin, its forward run's time steps"""
    from oracle.oracle import OracleDomain
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    import adjoint_case as case
    s0 = OracleDomain(nx, 11)
    e, _ = case.initial_energy(s0.field("e").copy(), nx, 200)
    b = OracleDomain(nx, 11)
    b.field("e")[:] = e
    b.dt_record(ncyc)
    assert b.step(ncyc) == 0
    return e, b.dt_recorded(ncyc), b


def test_tape_record_and_replay_reproduce_the_plain_cycle(oracle_built):
    """The decision tape changes nothing at the recorded point: the tape
    build recording, and a second domain replaying the recording, both give
    the parity build's fields bit for bit."""
    from oracle.oracle import OracleDomain, NODE_FIELDS, ELEM_FIELDS
    e, dts, plain = _noisy_case({})
    rec = OracleDomain(10, 11, tape=True)
    rec.field("e")[:] = e
    rec.dt_freeze(dts)
    rec.tape_record(len(dts))
    assert rec.step(len(dts)) == 0
    rep = OracleDomain(10, 11, tape=True)
    rep.field("e")[:] = e
    rep.dt_freeze(dts)
    rep.tape_replay(rec)
    assert rep.step(len(dts)) == 0
    for f in NODE_FIELDS + ELEM_FIELDS:
        assert np.array_equal(plain.field(f), rec.field(f)), f
        assert np.array_equal(plain.field(f), rep.field(f)), f
    with pytest.raises(RuntimeError):
        OracleDomain(10, 11).tape_record(5)        # the parity build has no tape


def test_tape_replay_holds_the_recorded_branches(oracle_built):
    """Away from the recorded point a replay keeps the recorded decisions.
    A cold element of the set-up field (e = 0, so p = 0: no pmin clamp) is
    given e = -1: the plain cycle clamps its pressure to pmin = 0, the
    replay keeps the recorded branch p = bvc * e < 0."""
    from oracle.oracle import OracleDomain
    k = 10 ** 3 - 1                                  # far corner, cold for many cycles
    rec = OracleDomain(10, 11, tape=True)
    e = rec.field("e").copy()
    rec.tape_record(1)
    assert rec.step(1) == 0
    dts = [rec.scalar("deltatime")]
    runs = {}
    for mode in ("plain", "replay"):
        d = OracleDomain(10, 11, tape=True)
        d.field("e")[:] = e
        d.field("e")[k] = -1.0
        d.dt_freeze(dts)
        if mode == "replay":
            d.tape_replay(rec)
        assert d.step(1) == 0
        runs[mode] = d.field("p")[k]
    assert runs["plain"] == 0.0
    assert runs["replay"] < 0.0


def test_extended_precision_build(oracle_built):
    """The long double tape build: the same problem to rounding of double
    precision, and its own recording replays bit for bit."""
    from oracle.oracle import OracleDomain
    e, dts, plain = _noisy_case({}, ncyc=20)
    rec = OracleDomain(10, 11, extended=True)
    assert rec.field("e").dtype == np.longdouble
    rec.field("e")[:] = e
    rec.dt_freeze(dts)
    rec.tape_record(len(dts))
    assert rec.step(len(dts)) == 0
    rep = OracleDomain(10, 11, extended=True)
    rep.field("e")[:] = e
    rep.dt_freeze(dts)
    rep.tape_replay(rec)
    assert rep.step(len(dts)) == 0
    assert np.array_equal(rec.field("e"), rep.field("e"))
    ef, el = plain.field("e"), rec.field("e").astype(np.float64)
    assert np.max(np.abs(el - ef)) <= 1e-12 * np.max(np.abs(ef))
