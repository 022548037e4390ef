"""The GPU halo kernels (lg_halo_pack / lg_halo_unpack) on one GPU: every rank
of a tp^3 decomposition is emulated by its own device arrays and buffers,
messages move between the ranks' device buffers by device-to-device copies
(the place MPI, NCCL or peer copies take on a multi-GPU system), and the
result is compared bit for bit with the reference's own exchange (the fixture
of tests/golden/make_halo_golden.py) and with the restatement
(oracle/halo_oracle.py) at larger sizes."""
import os

import numpy as np
import pytest

from halolib import CALL_SITES, KIND_ID, random_fields

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "halo_tp2_nx3.npz")


def _bits(a):
    return np.ascontiguousarray(a).view(np.int64)


def gpu_exchange(kind, nx, tp, nf, host_fields):
    """Pack on the GPU, move the messages device to device, unpack on the GPU.
    Returns (fields after, send buffers) as numpy."""
    import torch
    import lulesh_gb300 as lg
    nr = tp ** 3
    plans = [lg.HaloPlan(kind, nx, tp, r, nf) for r in range(nr)]
    dev = [[torch.from_numpy(a).cuda() for a in fl] for fl in host_fields]
    send = [torch.full((p.info()["buffer_doubles"],), float("nan"), dtype=torch.float64,
                       device="cuda") for p in plans]
    recv = [torch.zeros_like(s) for s in send]
    for r, p in enumerate(plans):
        p.pack(dev[r], send[r])
    smsgs = [p.messages("send") for p in plans]
    for r, p in enumerate(plans):
        for m in p.messages("recv"):
            src = [s for s in smsgs[m["peer"]] if s["peer"] == r]
            assert len(src) == 1
            n = nf * m["count"]
            recv[r][m["offset"]:m["offset"] + n].copy_(
                send[m["peer"]][src[0]["offset"]:src[0]["offset"] + n])
    for r, p in enumerate(plans):
        p.unpack(dev[r], recv[r])
    torch.cuda.synchronize()
    out = [[t.cpu().numpy() for t in fl] for fl in dev]
    for p in plans:
        p.close()
    return out, [s.cpu().numpy() for s in send], smsgs


@pytest.mark.parametrize("site", sorted(CALL_SITES))
def test_gpu_exchange_matches_reference_fixture(native_lib, site):
    g = np.load(GOLDEN)
    tp, nx = int(g["tp"]), int(g["nx"])
    kind, nf = CALL_SITES[site]
    nr = tp ** 3
    fin = [[g[f"{site}_in_r{r}_f{f}"].copy() for f in range(nf)] for r in range(nr)]
    out, _, _ = gpu_exchange(kind, nx, tp, nf, fin)
    for r in range(nr):
        for f in range(nf):
            assert np.array_equal(_bits(out[r][f]), _bits(g[f"{site}_out_r{r}_f{f}"])), (r, f)


@pytest.mark.parametrize("site", sorted(CALL_SITES))
@pytest.mark.parametrize("tp,nx", [(2, 16), (3, 7), (1, 5)])
def test_gpu_exchange_matches_restatement(native_lib, site, tp, nx):
    from oracle import halo_oracle as ho
    kind, nf = CALL_SITES[site]
    fields = random_fields(kind, nx, tp, nf, seed=tp * 100 + nx)
    want = [[a.copy() for a in fl] for fl in fields]
    ho.exchange(KIND_ID[kind], nx, tp, want)
    out, send, smsgs = gpu_exchange(kind, nx, tp, nf, fields)
    for r in range(tp ** 3):
        # every packed message equals the reference's packing of the fields
        ref_send = ho.pack(KIND_ID[kind], nx, tp, r, fields[r])
        for m in smsgs[r]:
            s = slice(m["offset"], m["offset"] + nf * m["count"])
            assert np.array_equal(_bits(send[r][s]), _bits(ref_send[s])), (r, m["peer"])
        for f in range(nf):
            assert np.array_equal(_bits(out[r][f]), _bits(want[r][f])), (r, f)


def test_gpu_exchange_deterministic(native_lib):
    kind, nf = CALL_SITES["forces"]
    fields = random_fields(kind, 12, 2, nf, seed=9)
    a, _, _ = gpu_exchange(kind, 12, 2, nf, [[x.copy() for x in fl] for fl in fields])
    b, _, _ = gpu_exchange(kind, 12, 2, nf, [[x.copy() for x in fl] for fl in fields])
    for r in range(8):
        for f in range(nf):
            assert np.array_equal(_bits(a[r][f]), _bits(b[r][f]))
