"""The no-allocation force entry point, checked against the regular path and
the oracle.

lg_calc_force_for_nodes_noalloc serves callers that keep every device buffer
themselves and cannot let the library allocate: codes that carve all device
memory from one pool sized at start-up, processes under a hard GPU memory
budget, and step loops that cannot afford cudaFree's device-wide
synchronisation.  This test plays such a caller: it holds the mesh state in
its own device buffers, calls the entry point twice in a row, and compares
the nodal forces with those the regular path (lg_create + lg_phase) and the
oracle (LagrangeNodal of the C restatement) compute from the same state.  It
also checks the VolumeError return and a call with no hourglass term made
right after one with it, since every call shares one scratch array.  The file
name sorts last so that a run stopping at the first failure has run every
other test before this one.
"""
import ctypes

import numpy as np
import pytest

from paritylib import FP64_TOL, field_rel_err

pytestmark = pytest.mark.gpu

NODE_IN = ["x", "y", "z", "xd", "yd", "zd"]
ELEM_IN = ["p", "q", "v", "volo", "ss", "elemMass"]
TOPO = ["nodelist", "nodeElemStart", "nodeElemCornerList"]
FORCES = ("fx", "fy", "fz")


def _bind(lib):
    f = lib.lg_calc_force_for_nodes_noalloc
    f.restype = ctypes.c_int
    f.argtypes = ([ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 3 +
                  [ctypes.c_void_p] * 12 + [ctypes.c_double] + [ctypes.c_void_p] * 3 +
                  [ctypes.c_void_p])
    lib.lg_last_error.restype = ctypes.c_char_p
    return f


class Caller:
    """A caller that owns its device buffers (torch tensors) and passes raw
    device pointers through the C ABI."""

    def __init__(self, lib, host: dict):
        import torch
        self.torch = torch
        self.call = _bind(lib)
        self.lib = lib
        self.E = host["p"].size
        self.N = host["x"].size
        self.dev = {f: torch.from_numpy(np.ascontiguousarray(a)).to("cuda")
                    for f, a in host.items()}
        self.out = {c: torch.empty(self.N, dtype=torch.float64, device="cuda") for c in FORCES}

    def forces(self, hgcoef: float):
        for t in self.out.values():
            t.fill_(float("nan"))
        self.torch.cuda.synchronize()
        st = self.call(self.E, self.N, *(self.dev[f].data_ptr() for f in TOPO),
                       *(self.dev[f].data_ptr() for f in NODE_IN + ELEM_IN), hgcoef,
                       *(self.out[c].data_ptr() for c in FORCES), None)
        return st, {c: self.out[c].cpu().numpy() for c in FORCES}


@pytest.fixture(scope="module")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _state(d):
    return {f: d.field(f) for f in NODE_IN + ELEM_IN + TOPO}


def test_noalloc_forces_match_regular_path(native_lib, cuda):
    import lulesh_gb300 as lg
    d = lg.Domain(12, 11, 1, 1)
    assert d.step(7) == 0
    caller = Caller(native_lib, _state(d))
    hg = d.scalar("hgcoef")
    # regular path: LagrangeNodal on the same state writes fx, fy, fz
    assert d.phase(1) == 0
    want = {c: d.field(c) for c in FORCES}
    for _ in range(2):
        st, got = caller.forces(hg)
        assert st == 0, native_lib.lg_last_error()
        for c in FORCES:
            assert np.all(np.isfinite(got[c])), c
            assert field_rel_err(got[c], want[c]) <= FP64_TOL, c


def test_noalloc_forces_match_oracle(native_lib, oracle_built, cuda):
    """The oracle's state after 7 cycles of s=12 r11 goes in; the oracle's own
    LagrangeNodal forces of that state are the expected output."""
    from oracle.oracle import OracleDomain
    o = OracleDomain(12, 11, 1, 1)
    assert o.step(7) == 0
    caller = Caller(native_lib, {f: o.field(f).copy() for f in NODE_IN + ELEM_IN + TOPO})
    assert o.phase(1) == 0
    want = {c: o.field(c).copy() for c in FORCES}
    for _ in range(2):
        st, got = caller.forces(o.scalar("hgcoef"))
        assert st == 0, native_lib.lg_last_error()
        for c in FORCES:
            assert field_rel_err(got[c], want[c]) <= FP64_TOL, c
    o.close()


def test_noalloc_without_hourglass_after_a_call_with_it(native_lib, cuda):
    """hgcoef = 0 skips the hourglass corner forces; the shared scratch still
    holds the previous call's, and they must not leak into the sums."""
    import lulesh_gb300 as lg
    d = lg.Domain(10, 11, 1, 1)
    assert d.step(9) == 0
    caller = Caller(native_lib, _state(d))
    st, with_hg = caller.forces(3.0)
    assert st == 0, native_lib.lg_last_error()
    d.set_scalar("hgcoef", 0.0)
    assert d.phase(1) == 0
    want = {c: d.field(c) for c in FORCES}
    for _ in range(2):
        st, got = caller.forces(0.0)
        assert st == 0, native_lib.lg_last_error()
        for c in FORCES:
            assert field_rel_err(got[c], want[c]) <= FP64_TOL, c
    # and the hourglass term was really there before
    assert max(np.max(np.abs(with_hg[c] - want[c])) for c in FORCES) > 0.0


def test_noalloc_reports_volume_error(native_lib, cuda):
    """A non-positive relative volume, planted on the host before upload,
    gives -1 (the reference's exit(VolumeError)); the next clean call on the
    same shared status word gives 0 again."""
    import lulesh_gb300 as lg
    d = lg.Domain(6, 3, 1, 1)
    assert d.step(3) == 0
    host = _state(d)
    bad = dict(host)
    bad["v"] = host["v"].copy()
    bad["v"][5] = -1.0
    st, _ = Caller(native_lib, bad).forces(3.0)
    assert st == -1
    st, _ = Caller(native_lib, host).forces(3.0)
    assert st == 0, native_lib.lg_last_error()


def test_noalloc_rejects_meshes_beyond_its_scratch(native_lib):
    call = _bind(native_lib)
    dummy = ctypes.c_void_p(1)  # never dereferenced: the size check comes first
    st = call(32769, 1000, *([dummy] * 15), 3.0, dummy, dummy, dummy, None)
    assert st == 1  # LG_ERR_INVALID
    assert b"32768" in native_lib.lg_last_error()
