"""Device-side set-up (lg_setup.cu) against the host set-up.

The host set-up (lg_problem.cc, build_sedov) is pinned to the reference's
Domain::Domain by the oracle's golden set-up digests; a host-only handle
(device=-1) serves it.  A device handle builds the mesh, the fields and the
corner lists with kernels; every double field, integer array and time-step
scalar must equal the host set-up's bit for bit.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

I32_FIELDS = ["nodelist", "lxim", "lxip", "letam", "letap", "lzetam", "lzetap", "elemBC",
              "regNumList", "regElemSize", "symmX", "symmY", "symmZ", "nodeElemStart",
              "nodeElemCornerList"]
SCALARS = ["time", "deltatime", "dtcourant", "dthydro", "stoptime", "dtmax", "dtfixed",
           "deltatimemultlb", "deltatimemultub", "hgcoef", "cycle", "numElem", "numNode"]

CASES = [  # nx, numReg, balance, cost, hgcoef, einit_factor
    (1, 1, 1, 1, 3.0, 1.0), (2, 3, 1, 1, 3.0, 1.0), (3, 11, 1, 1, 3.0, 1.0),
    (7, 5, 2, 3, 1.7, 0.6), (16, 16, 2, 4, 3.0, 1.0), (45, 11, 1, 1, 3.0, 1.0),
    (64, 4, 1, 2, 2.2, 1.9)]


def _same_bits(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if a.dtype == np.float64:
        return a.shape == b.shape and np.array_equal(a.view(np.int64), b.view(np.int64))
    return np.array_equal(a, b)


@pytest.mark.parametrize("case", CASES)
def test_device_setup_equals_host_setup(native_lib, case):
    import lulesh_gb300 as lg
    nx, nr, b, c, hg, ef = case
    host = lg.Domain(nx, nr, b, c, hgcoef=hg, einit_factor=ef, device=-1)
    dev = lg.Domain(nx, nr, b, c, hgcoef=hg, einit_factor=ef)
    for f in lg.NODE_FIELDS + lg.ELEM_FIELDS:
        assert _same_bits(host.field(f), dev.field(f)), f
    for s in SCALARS:
        assert host.scalar(s) == dev.scalar(s), s
    for f in I32_FIELDS:
        assert _same_bits(host.field(f), dev.field(f)), f


def test_device_setup_runs_like_host_setup(native_lib):
    """Topology read back to the host, then the cycle: the same run either way."""
    import lulesh_gb300 as lg
    a = lg.Domain(20, 11, its=50)
    b = lg.Domain(20, 11, its=50)
    b.field("nodeElemCornerList")  # download the device-built topology first
    assert a.run() == 0 and b.run() == 0
    for f in lg.NODE_FIELDS + lg.ELEM_FIELDS:
        assert _same_bits(a.field(f), b.field(f)), f


def test_reset_restores_the_setup_state(native_lib):
    import lulesh_gb300 as lg
    d = lg.Domain(24, 11)
    init = {f: d.field(f) for f in lg.NODE_FIELDS + lg.ELEM_FIELDS}
    assert d.step(30) == 0
    d.reset()
    assert d.scalar("cycle") == 0
    for f, v in init.items():
        assert _same_bits(v, d.field(f)), f
    # a replaced region map survives the reset; the fields return to set-up
    reg = d.field("regNumList")
    reg2 = reg.copy()
    reg2[reg2 == 1] = 2
    d.set_field("regNumList", reg2)
    assert d.step(5) == 0
    d.reset()
    assert np.array_equal(d.field("regNumList"), reg2)
    for f, v in init.items():
        assert _same_bits(v, d.field(f)), f


def _selfcheck(e, nx):
    """lulesh-util.cc:189-218, serially, in the reference's loop order"""
    e = [float(x) for x in e[: nx * nx]]
    max_abs = total = max_rel = 0.0
    for j in range(nx):
        for k in range(j + 1, nx):
            a = abs(e[j * nx + k] - e[k * nx + j])
            total += a
            if max_abs < a:
                max_abs = a
            den = e[k * nx + j]
            if den != 0.0:
                r = a / den
            else:  # IEEE: 0/0 is NaN, a/(+-0) is +-inf
                r = float("nan") if a == 0.0 else math.copysign(float("inf"), den)
            if max_rel < r:
                max_rel = r
    return e[0], max_abs, total, max_rel


@pytest.mark.parametrize("nx,cycles", [(1, 3), (30, 100), (150, 40)])
def test_device_selfcheck_equals_serial_loop(native_lib, nx, cycles):
    import lulesh_gb300 as lg
    d = lg.Domain(nx, 11, its=cycles)
    assert d.run() == 0
    v = d.verify()
    ref = _selfcheck(d.field("e"), nx)
    got = (v["origin_energy"], v["MaxAbsDiff"], v["TotalAbsDiff"], v["MaxRelDiff"])
    assert got == ref, (got, ref)
