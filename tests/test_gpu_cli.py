"""The drop-in command line on the device: the report against the reference
executable's (tests/golden/report.json), the progress lines, and the VTK
viz dump against the library's own fields."""
import json
import os
import re
import struct
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "lulesh_gb300", "bin", "lulesh_gpu")
GOLDEN = json.load(open(os.path.join(ROOT, "tests", "golden", "report.json")))


def _report(text):
    grab = lambda key: re.search(key + r"\s*=\s*(\S+)", text).group(1)  # noqa: E731
    return {"cycles": int(grab("Iteration count")), "origin_energy": grab("Final Origin Energy"),
            "MaxAbsDiff": grab("MaxAbsDiff"), "TotalAbsDiff": grab("TotalAbsDiff"),
            "MaxRelDiff": grab("MaxRelDiff")}


@pytest.mark.parametrize("label", ["s8_i100", "s16_r16_b2_c4_i60", "s30_stoptime"])
def test_cli_report_matches_reference(native_lib, label):
    g = GOLDEN[label]
    r = subprocess.run([CLI] + g["args"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    rep = _report(r.stdout)
    assert rep["cycles"] == g["cycles"]
    assert rep["origin_energy"] == g["origin_energy"]
    # the symmetry deltas are rounding-level: their magnitude, not their digits
    for k in ("MaxAbsDiff", "TotalAbsDiff", "MaxRelDiff"):
        assert float(rep[k]) <= 10 * max(float(g[k]), 1e-300), (k, rep[k], g[k])


def test_cli_progress_lines(native_lib):
    r = subprocess.run([CLI, "-s", "6", "-i", "12", "-p"], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0
    lines = [l for l in r.stdout.splitlines() if l.startswith("cycle = ")]
    assert len(lines) == 12 and lines[-1].startswith("cycle = 12, time = ")


def _read_vtk(path):
    data = open(path, "rb").read()
    pos = 0

    def line():
        nonlocal pos
        end = data.index(b"\n", pos)
        s = data[pos:end].decode()
        pos = end + 1
        return s

    def block(count, fmt):
        nonlocal pos
        size = struct.calcsize(">" + fmt)
        arr = np.frombuffer(data[pos:pos + count * size], dtype=">" + fmt)
        pos += count * size
        return arr

    out = {}
    while pos < len(data):
        s = line()
        if s.startswith("POINTS"):
            n, typ = int(s.split()[1]), s.split()[2]
            out["points_type"] = typ
            out["points"] = block(3 * n, {"double": "d", "float": "f"}[typ]).reshape(n, 3)
        elif s.startswith("LULESH cycle"):
            out["cycle"], out["time"] = int(s.split()[2]), float(s.split()[4])
        elif s.startswith("CELLS "):
            n, size = map(int, s.split()[1:3])
            out["cells"] = block(size, "i").reshape(n, 9)
        elif s.startswith("CELL_TYPES"):
            out["types"] = block(int(s.split()[1]), "i")
        elif s.startswith("CELL_DATA"):
            out["ncell"] = int(s.split()[1])
        elif s.startswith("POINT_DATA"):
            out["npoint"] = int(s.split()[1])
        elif s.startswith("SCALARS"):
            name, typ = s.split()[1:3]
            out.setdefault("scalars", []).append((name, typ))
            line()  # LOOKUP_TABLE
            n = out["npoint"] if "npoint" in out else out["ncell"]
            out[name] = block(n, {"double": "d", "float": "f", "int": "i"}[typ])
    return out


# The variables DumpDomainToVisit writes, in its order, with their types and
# centring (lulesh-viz.cc:171-252): the region material, then DB_FLOAT zone
# variables e, p, v, q, then DB_FLOAT node variables speed, xd, yd, zd.  Its
# mesh coordinates are DB_FLOAT too (:150-165).
VIZ_VARIABLES = [("regions", "int"), ("e", "float"), ("p", "float"), ("v", "float"),
                 ("q", "float"), ("speed", "float"), ("xd", "float"), ("yd", "float"),
                 ("zd", "float")]


def test_cli_vtk_dump(native_lib, tmp_path):
    import lulesh_gb300 as lg
    path = str(tmp_path / "sedov.vtk")
    r = subprocess.run([CLI, "-s", "5", "-i", "20", "-q", "--viz-vtk", path],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout
    v = _read_vtk(path)
    assert v["scalars"] == VIZ_VARIABLES
    assert v["points_type"] == "float"
    d = lg.Domain(5, 11, its=20)
    assert d.run() == 0
    assert v["cycle"] == 20 and v["time"] == float("%.9e" % d.scalar("time"))
    f32 = lambda name: d.field(name).astype(np.float32)
    for k, name in enumerate("xyz"):
        assert np.array_equal(v["points"][:, k], f32(name)), name
    assert np.array_equal(v["cells"][:, 1:].ravel(), d.field("nodelist"))
    assert np.all(v["cells"][:, 0] == 8) and np.all(v["types"] == 12)
    assert np.array_equal(v["regions"], d.field("regNumList"))
    assert v["regions"].min() >= 1 and v["regions"].max() <= 11  # region numbers from 1
    for name in ("e", "p", "v", "q", "xd", "yd", "zd"):
        assert np.array_equal(v[name], f32(name)), name
    xd, yd, zd = f32("xd"), f32("yd"), f32("zd")
    sp = np.sqrt(xd * xd + yd * yd + zd * zd)
    assert np.allclose(v["speed"], sp, rtol=1e-6, atol=0)
