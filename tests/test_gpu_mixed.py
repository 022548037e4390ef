"""Mixed precision (FP32 stress, hourglass, kinematics and Q; FP64 state,
volume, EOS and dt) against the FP64 path on the same problem.

The bar (stated by the benchmark spec): origin energy within 1e-5 relative of the FP64
run.  Also checked: total energy (internal sum(e*volo) plus kinetic
sum(m|u|^2)/2) within 1e-5, the same cycle count to stoptime, and symmetry
deltas that stay small (they are rounding-level in FP64 and FP32-level here).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def total_energy(d):
    m = d.field("nodalMass")
    ke = 0.5 * np.sum(m * (d.field("xd") ** 2 + d.field("yd") ** 2 + d.field("zd") ** 2))
    return float(np.sum(d.field("e") * d.field("volo")) + ke)


def _run(lg, case, precision):
    nx, nr, b, c, its = case
    d = lg.Domain(nx, nr, b, c, its=its, precision=precision)
    st = d.run()
    out = {"st": st, "cycle": d.cycle, "verify": d.verify(), "total": total_energy(d),
           "e": d.field("e")}
    d.close()
    return out


@pytest.mark.parametrize("case", [(30, 11, 1, 1, 100), (48, 11, 1, 1, 200), (64, 16, 2, 4, 300),
                                  (30, 11, 1, 1, 9999999)])
def test_mixed_energy_error_vs_fp64(native_lib, case):
    import lulesh_gb300 as lg
    m = _run(lg, case, "mixed")
    f = _run(lg, case, "fp64")
    assert m["st"] == 0 and f["st"] == 0
    assert m["cycle"] == f["cycle"]
    e0m, e0f = m["verify"]["origin_energy"], f["verify"]["origin_energy"]
    assert abs(e0m / e0f - 1) <= 1e-5
    assert abs(m["total"] / f["total"] - 1) <= 1e-5
    # symmetry of plane 0 stays at FP32 rounding level
    assert m["verify"]["MaxRelDiff"] <= 1e-4
    assert np.max(np.abs(m["e"] - f["e"])) <= 1e-4 * np.max(np.abs(f["e"]))


def test_mixed_gradient_temporaries_not_exposed_as_fp64(native_lib):
    import lulesh_gb300 as lg
    d = lg.Domain(8, its=2, precision="mixed")
    assert d.run() == 0
    with pytest.raises(lg.LuleshError):
        d.field("delv_xi")
    d.field("delv")  # the FP64 relative-volume change is still an FP64 field


def test_mixed_deterministic(native_lib):
    import lulesh_gb300 as lg
    a = _run(lg, (20, 11, 1, 1, 50), "mixed")["e"]
    b = _run(lg, (20, 11, 1, 1, 50), "mixed")["e"]
    assert np.array_equal(a.view(np.int64), b.view(np.int64))
