"""The C ABI from a compiled C program (tests/abi_smoke.c), with no Python in
the call path: the same create / run / verify / report / field calls a C or
C++ host makes, checked against the reference's golden report values and
field dumps, plus the field-sync integration pattern (every field up, one
cycle, every field down) against a resident run, bit for bit."""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from paritylib import FP64_TOL, compare_states

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
NODE = ["x", "y", "z", "xd", "yd", "zd", "xdd", "ydd", "zdd", "fx", "fy", "fz", "nodalMass"]
ELEM = ["e", "p", "q", "ql", "qq", "v", "volo", "vnew", "delv", "vdov", "arealg", "ss",
        "elemMass"]


@pytest.fixture(scope="module")
def abi_smoke(native_lib, tmp_path_factory):
    """Compile abi_smoke.c as C99 with warnings as errors and link it to the
    library through -l, with an rpath, as a host program would."""
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    from lulesh_gb300 import build
    libdir = os.path.dirname(build.LIB)
    exe = str(tmp_path_factory.mktemp("abi") / "abi_smoke")
    subprocess.run([cc, "-std=c99", "-O2", "-Wall", "-Wextra", "-Werror",
                    "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "abi_smoke.c"),
                    "-L", libdir, "-llulesh_gb300", "-Wl,-rpath," + libdir, "-o", exe],
                   check=True)
    return exe


def test_c_caller_compiles_and_links(abi_smoke):
    r = subprocess.run([abi_smoke], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr


def _run(exe, args, tmp_path):
    r = subprocess.run([exe, "run"] + [str(a) for a in args] + [str(tmp_path)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    out = r.stdout
    kv = dict(re.findall(r"^(status|cycle|time) (\S+)$", out, re.M))
    ver = [float(v) for v in re.search(r"^verify (.*)$", out, re.M).group(1).split()]
    report = out.split("--- report\n", 1)[1].split("--- end", 1)[0]
    fields = {f: np.fromfile(os.path.join(tmp_path, f + ".f64"), dtype=np.float64)
              for f in NODE + ELEM}
    return kv, ver, report, fields


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp64-fma"])
@pytest.mark.parametrize("fname", sorted(f for f in os.listdir(GOLDEN) if f.startswith("fields_")))
def test_c_caller_fields_match_reference_golden(abi_smoke, tmp_path, fname, precision):
    g = np.load(os.path.join(GOLDEN, fname))
    nx, nr, b, c, cyc = (int(v) for v in g["case"])
    hg, ef = (float(v) for v in g["params"])
    if hg != 3.0 or ef != 1.0:
        pytest.skip("the C caller builds the reference's own problem (hgcoef 3, energy x1)")
    kv, _, _, fields = _run(abi_smoke, [nx, nr, b, c, cyc, precision], tmp_path)
    assert int(kv["status"]) == 0 and int(kv["cycle"]) == int(g["cycle"])
    errs = compare_states(fields, g, NODE + ELEM)
    assert max(errs.values()) <= FP64_TOL, errs


@pytest.mark.gpu
@pytest.mark.parametrize("label", ["s8_i100", "s16_r16_b2_c4_i60"])
def test_c_caller_report_matches_reference(abi_smoke, tmp_path, label):
    import json
    rep = json.load(open(os.path.join(GOLDEN, "report.json")))[label]
    a = {"-s": 30, "-r": 11, "-b": 1, "-c": 1, "-i": 9999999}
    for i in range(0, len(rep["args"]), 2):
        a[rep["args"][i]] = int(rep["args"][i + 1])
    kv, ver, report, _ = _run(abi_smoke, [a["-s"], a["-r"], a["-b"], a["-c"], a["-i"], "fp64"],
                              tmp_path)
    assert int(kv["cycle"]) == rep["cycles"]
    assert "%.6e" % ver[0] == rep["origin_energy"]
    assert "Final Origin Energy =  %12s" % rep["origin_energy"] in report
    assert "Iteration count     =  %d" % rep["cycles"] in report
    for k, v in zip(("MaxAbsDiff", "TotalAbsDiff"), ver[1:3]):
        assert v <= 10 * float(rep[k]) + 1e-12 * abs(ver[0])


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp64-fma", "mixed"])
def test_c_caller_field_sync_pattern(abi_smoke, precision):
    r = subprocess.run([abi_smoke, "sync", "16", "16", "2", "4", "10", precision],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "cycles 10 10" in r.stdout
    assert "sync-equal 1" in r.stdout, r.stdout
