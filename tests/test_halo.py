"""Halo pack/unpack plans (lg_halo_*) on the CPU.

Three layers, each checked bit for bit:
  * the restatement (oracle/halo_oracle.py) against the reference's own
    CommRecv / CommSend / CommSBN / CommSyncPosVel / CommMonoQ, run for every
    rank of a tp^3 decomposition in one process (oracle/halo_ref_driver.cc;
    where the reference sources are present);
  * the library's plans (message peers, lengths, offsets and value lists)
    against the restatement, applied on the CPU from the plan's own lists;
  * the same exchange split over two gloo processes on 127.0.0.1, each owning
    half of the ranks, messages moved by torch.distributed send/recv as the
    reference moves them by MPI_Isend/MPI_Irecv.
The GPU kernels themselves are checked in tests/test_gpu_halo.py.
"""
import ctypes
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

from halolib import (CALL_SITES, KIND_ID, cpu_pack, cpu_unpack, random_fields, transport)

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HALO_REF = os.path.join(ROOT, "oracle", "_ref", "liblulesh_halo_ref.so")
REF_NAMES = {"forces": ["fx", "fy", "fz"], "pos_vel": ["x", "y", "z", "xd", "yd", "zd"],
             "monoq": ["delv_xi", "delv_eta", "delv_zeta"], "nodal_mass": ["nodalMass"]}
REF_KIND = {"forces": 0, "pos_vel": 1, "monoq": 2, "nodal_mass": 3}


def _bits(a):
    return np.ascontiguousarray(a).view(np.int64)


@pytest.fixture(scope="module")
def halo_ref(oracle_built):
    if not os.path.exists(HALO_REF):
        pytest.skip("reference sources not available on this host")
    lib = ctypes.CDLL(HALO_REF)
    lib.hr_create.argtypes = [ctypes.c_int, ctypes.c_int]
    P = ctypes.POINTER(ctypes.c_double)
    for f in ("hr_field",):
        getattr(lib, f).restype = P
        getattr(lib, f).argtypes = [ctypes.c_int, ctypes.c_char_p,
                                    ctypes.POINTER(ctypes.c_size_t)]
    for f in ("hr_send_buffer", "hr_recv_buffer"):
        getattr(lib, f).restype = P
        getattr(lib, f).argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_size_t)]
    lib.hr_exchange.argtypes = [ctypes.c_int]
    return lib


def _arr(p, n):
    return np.ctypeslib.as_array(p, shape=(n,))


@pytest.mark.parametrize("site", sorted(CALL_SITES))
@pytest.mark.parametrize("tp,nx", [(2, 3), (2, 6), (3, 4)])
def test_restatement_matches_reference_exchange(halo_ref, site, tp, nx):
    from oracle import halo_oracle as ho
    kind, nf = CALL_SITES[site]
    nr = halo_ref.hr_create(tp, nx)
    if site == "monoq":
        halo_ref.hr_alloc_gradients()
    rng = np.random.default_rng(11)
    mine = []
    for r in range(nr):
        fl = []
        for name in REF_NAMES[site]:
            n = ctypes.c_size_t()
            a = _arr(halo_ref.hr_field(r, name.encode(), ctypes.byref(n)), n.value)
            a[:] = rng.standard_normal(n.value)
            fl.append(a.copy())
        mine.append(fl)
    before = [[a.copy() for a in fl] for fl in mine]
    halo_ref.hr_exchange(REF_KIND[site])
    recv = ho.exchange(KIND_ID[kind], nx, tp, mine)
    for r in range(nr):
        for name, m in zip(REF_NAMES[site], mine[r]):
            n = ctypes.c_size_t()
            a = _arr(halo_ref.hr_field(r, name.encode(), ctypes.byref(n)), n.value)
            assert np.array_equal(_bits(a), _bits(m)), (r, name)
        n = ctypes.c_size_t()
        rb = _arr(halo_ref.hr_recv_buffer(r, ctypes.byref(n)), n.value)
        assert n.value == ho.buffer_doubles(nx, tp, r)
        for msg in ho.messages(KIND_ID[kind], nx, tp, r, nf, "recv"):
            s = slice(msg["offset"], msg["offset"] + nf * msg["count"])
            assert np.array_equal(_bits(rb[s]), _bits(recv[r][s])), (r, msg["peer"])
        # the reference's send buffer holds every message as CommSend packed
        # it, from the fields before the exchange
        sb = _arr(halo_ref.hr_send_buffer(r, ctypes.byref(n)), n.value)
        mysend = ho.pack(KIND_ID[kind], nx, tp, r, before[r])
        for msg in ho.messages(KIND_ID[kind], nx, tp, r, nf, "send"):
            s = slice(msg["offset"], msg["offset"] + nf * msg["count"])
            assert np.array_equal(_bits(sb[s]), _bits(mysend[s])), (r, msg["peer"])


@pytest.mark.parametrize("site", sorted(CALL_SITES))
@pytest.mark.parametrize("tp,nx", [(1, 3), (2, 1), (2, 4), (3, 2), (3, 3)])
def test_plans_match_restatement(native_lib, site, tp, nx):
    """Message lists, buffer sizes and a whole exchange applied on the CPU
    from the plans' own value lists."""
    import lulesh_gb300 as lg
    from oracle import halo_oracle as ho
    kind, nf = CALL_SITES[site]
    k = KIND_ID[kind]
    plans = [lg.HaloPlan(kind, nx, tp, r, nf) for r in range(tp ** 3)]
    for r, p in enumerate(plans):
        info = p.info()
        assert info["buffer_doubles"] == ho.buffer_doubles(nx, tp, r)
        for side in ("send", "recv"):
            want = [(m["peer"], m["count"], m["offset"])
                    for m in ho.messages(k, nx, tp, r, nf, side)]
            got = [(m["peer"], m["count"], m["offset"]) for m in p.messages(side)]
            assert got == want, (r, side)
    fields = random_fields(kind, nx, tp, nf, seed=3)
    want = [[a.copy() for a in fl] for fl in fields]
    ho.exchange(k, nx, tp, want)
    send = [np.zeros(p.info()["buffer_doubles"]) for p in plans]
    recv = [np.zeros(p.info()["buffer_doubles"]) for p in plans]
    for r, p in enumerate(plans):
        cpu_pack(p.entries("send"), fields[r], send[r])
    transport([p.messages("send") for p in plans], [p.messages("recv") for p in plans],
              send, recv, nf)
    for r, p in enumerate(plans):
        cpu_unpack(kind, p.entries("recv"), fields[r], recv[r])
        for f in range(nf):
            assert np.array_equal(_bits(fields[r][f]), _bits(want[r][f])), (r, f)


def test_plan_rejects_bad_arguments(native_lib):
    import lulesh_gb300 as lg
    for args in [(5, 4, 2, 0, 3), (0, 0, 2, 0, 3), (0, 4, 2, 8, 3), (0, 4, 2, 0, 7),
                 (0, 4, 0, 0, 3)]:
        with pytest.raises(lg.LuleshError):
            lg.HaloPlan(*args)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


RANK_SCRIPT = r'''
import json, os, sys
sys.path.insert(0, {root!r}); sys.path.insert(0, {tests!r})
import numpy as np, torch, torch.distributed as dist
import lulesh_gb300 as lg
from oracle import halo_oracle as ho
from halolib import CALL_SITES, KIND_ID, cpu_pack, cpu_unpack, random_fields
dist.init_process_group("gloo")
me, ws = dist.get_rank(), dist.get_world_size()
tp, nx = 2, 3
owner = lambda r: r % ws                    # domain rank r lives in process owner(r)
out = {{}}
for site in sorted(CALL_SITES):
    kind, nf = CALL_SITES[site]
    fields = random_fields(kind, nx, tp, nf, seed=5)
    want = [[a.copy() for a in fl] for fl in fields]
    ho.exchange(KIND_ID[kind], nx, tp, want)
    mine = [r for r in range(tp ** 3) if owner(r) == me]
    plans = {{r: lg.HaloPlan(kind, nx, tp, r, nf) for r in mine}}
    send = {{r: np.zeros(plans[r].info()["buffer_doubles"]) for r in mine}}
    recv = {{r: np.zeros(plans[r].info()["buffer_doubles"]) for r in mine}}
    for r in mine:
        cpu_pack(plans[r].entries("send"), fields[r], send[r])
    reqs, bufs = [], []
    # every message crosses with a tag naming its (sender, receiver) pair; a
    # message between two domains of the same process is copied directly
    for r in mine:
        for m in plans[r].messages("send"):
            seg = send[r][m["offset"]:m["offset"] + nf * m["count"]]
            if owner(m["peer"]) == me:
                continue
            reqs.append(dist.isend(torch.from_numpy(seg.copy()), owner(m["peer"]),
                                   tag=r * 64 + m["peer"]))
    for r in mine:
        for m in plans[r].messages("recv"):
            n = nf * m["count"]
            if owner(m["peer"]) == me:
                src = [s for s in plans[m["peer"]].messages("send") if s["peer"] == r][0]
                recv[r][m["offset"]:m["offset"] + n] = send[m["peer"]][src["offset"]:src["offset"] + n]
                continue
            t = torch.empty(n, dtype=torch.float64)
            reqs.append(dist.irecv(t, owner(m["peer"]), tag=m["peer"] * 64 + r))
            bufs.append((r, m["offset"], t))
    for q in reqs:
        q.wait()
    for r, off, t in bufs:
        recv[r][off:off + t.numel()] = t.numpy()
    ok = True
    for r in mine:
        cpu_unpack(kind, plans[r].entries("recv"), fields[r], recv[r])
        for f in range(nf):
            ok &= bool(np.array_equal(fields[r][f].view(np.int64), want[r][f].view(np.int64)))
    out[site] = ok
dist.barrier()
print(json.dumps({{"rank": me, "ok": out}}))
'''


def test_two_process_exchange_over_gloo(native_lib, tmp_path):
    """tp=2 (8 domain ranks) split over two gloo processes: each process packs
    its domains from the plans, sends each message to the process owning its
    peer, receives into the offsets the plans give, unpacks, and compares with
    the restatement's exchange of all 8 ranks."""
    pytest.importorskip("torch")
    script = tmp_path / "halo_rank.py"
    script.write_text(RANK_SCRIPT.format(root=ROOT, tests=os.path.join(ROOT, "tests")))
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, str(script)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=300)
        assert p.returncode == 0, e[-3000:]
        outs.append(o)
    import json
    for o in outs:
        res = json.loads(o.strip().splitlines()[-1])
        assert all(res["ok"].values()), res


GOLDEN = os.path.join(ROOT, "tests", "golden", "halo_tp2_nx3.npz")


def _golden_fields(g, site, io, nr, nf):
    return [[g[f"{site}_{io}_r{r}_f{f}"].copy() for f in range(nf)] for r in range(nr)]


@pytest.mark.parametrize("site", sorted(CALL_SITES))
def test_restatement_matches_reference_fixture(site):
    """The fixture of the reference's own exchange (tests/golden/make_halo_golden.py)."""
    from oracle import halo_oracle as ho
    g = np.load(GOLDEN)
    tp, nx = int(g["tp"]), int(g["nx"])
    kind, nf = CALL_SITES[site]
    fields = _golden_fields(g, site, "in", tp ** 3, nf)
    ho.exchange(KIND_ID[kind], nx, tp, fields)
    want = _golden_fields(g, site, "out", tp ** 3, nf)
    for r in range(tp ** 3):
        for f in range(nf):
            assert np.array_equal(_bits(fields[r][f]), _bits(want[r][f])), (r, f)
