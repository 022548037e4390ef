"""The no-allocation force entry point, checked against the regular path.

lg_calc_force_for_nodes_noalloc serves callers that keep every device buffer
themselves and cannot let the library allocate: codes that carve all device
memory from one pool sized at start-up, processes under a hard GPU memory
budget, and step loops that cannot afford cudaFree's device-wide
synchronisation.  This test plays such a caller: it holds the mesh state in
its own device buffers, calls the entry point twice in a row, and compares
the nodal forces with those the regular path (lg_create + lg_phase) computes
from the same state.  The file name sorts last so that a run stopping at the
first failure has run every other test before this one.
"""
import ctypes

import numpy as np
import pytest

from paritylib import FP64_TOL, field_rel_err

pytestmark = pytest.mark.gpu

NODE_IN = ["x", "y", "z", "xd", "yd", "zd"]
ELEM_IN = ["p", "q", "v", "volo", "ss", "elemMass"]
TOPO = ["nodelist", "nodeElemStart", "nodeElemCornerList"]


def _bind(lib):
    f = lib.lg_calc_force_for_nodes_noalloc
    f.restype = ctypes.c_int
    f.argtypes = ([ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 3 +
                  [ctypes.c_void_p] * 12 + [ctypes.c_double] + [ctypes.c_void_p] * 3 +
                  [ctypes.c_void_p])
    return f


def test_noalloc_forces_match_regular_path(native_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import lulesh_gb300 as lg
    call = _bind(native_lib)

    d = lg.Domain(12, 11, 1, 1)
    assert d.step(7) == 0
    E, N = d.numElem, d.numNode
    host = {f: d.field(f) for f in NODE_IN + ELEM_IN + TOPO}
    dev = {f: torch.from_numpy(np.ascontiguousarray(a)).to("cuda") for f, a in host.items()}
    hg = d.scalar("hgcoef")

    # regular path: LagrangeNodal on the same state writes fx, fy, fz
    assert d.phase(1) == 0
    want = {c: d.field(c) for c in ("fx", "fy", "fz")}

    out = {c: torch.empty(N, dtype=torch.float64, device="cuda") for c in ("fx", "fy", "fz")}
    for _ in range(2):
        for t in out.values():
            t.fill_(float("nan"))
        torch.cuda.synchronize()
        st = call(E, N, *(dev[f].data_ptr() for f in TOPO),
                  *(dev[f].data_ptr() for f in NODE_IN + ELEM_IN), hg,
                  out["fx"].data_ptr(), out["fy"].data_ptr(), out["fz"].data_ptr(), None)
        assert st == 0, native_lib.lg_last_error()
        for c in ("fx", "fy", "fz"):
            got = out[c].cpu().numpy()
            assert np.all(np.isfinite(got)), c
            assert field_rel_err(got, want[c]) <= FP64_TOL, c


def test_noalloc_rejects_meshes_beyond_its_scratch(native_lib):
    call = _bind(native_lib)
    native_lib.lg_last_error.restype = ctypes.c_char_p
    dummy = ctypes.c_void_p(1)  # never dereferenced: the size check comes first
    st = call(32769, 1000, *([dummy] * 15), 3.0, dummy, dummy, dummy, None)
    assert st == 1  # LG_ERR_INVALID
    assert b"32768" in native_lib.lg_last_error()
