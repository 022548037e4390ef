"""Restatement of the reference's halo exchange (lulesh-comm.cc) in numpy.

Test infrastructure only: the GPU halo kernels (lulesh_gb300/csrc/lg_halo.cu)
are checked against it, and it is checked against the reference's own
CommRecv / CommSend / CommSBN / CommSyncPosVel / CommMonoQ run for every rank
in one process (oracle/halo_ref_driver.cc, tests/test_halo.py).  Nothing in
the product imports it.

The reference decomposes the mesh into tp x tp x tp cubes of nx elements, one
per MPI rank (InitMeshDecomp, lulesh-init.cc:676-738: rank = col + row*tp +
plane*tp^2), and exchanges up to 26 messages per rank: 6 faces, 12 edges and
8 corners.  The table below transcribes, message by message and in the
reference's order, the condition under which a rank sends and receives it,
the neighbour, and the index formula of its values (CommRecv
lulesh-comm.cc:59-355, CommSend 357-845).  A message holds its fields one
after another (field fi at fi*count).  The buffer offset of a message is
pmsg*maxPlaneComm + emsg*maxEdgeComm + cmsg*16 doubles over the messages
before it of each class (faces, edges, corners).
"""
from __future__ import annotations

import numpy as np

PAD = 16  # CACHE_COHERENCE_PAD_REAL: 128 bytes of doubles (lulesh.h:98)
MAX_FIELDS = 6  # MAX_FIELDS_PER_MPI_COMM (lulesh.h:94)

SBN, SYNC_POS_VEL, MONOQ = 0, 1, 2


def cache_align(n: int) -> int:
    """CACHE_ALIGN_REAL (lulesh.h:100-101)."""
    return (n + PAD - 1) & ~(PAD - 1)


def location(rank: int, tp: int) -> tuple[int, int, int]:
    """(col, row, plane) of a rank (InitMeshDecomp, lulesh-init.cc:709-735)."""
    return rank % tp, (rank // tp) % tp, rank // (tp * tp)


def _table(tp, dx, dy, dz):
    """The 26 messages in the reference's order: (class, flags needed,
    send needs doSend, receive needs doRecv, peer rank offset, index list).
    flags: subset of 'rm rM cm cM pm pM' (rowMin ... planeMax)."""
    T2 = tp * tp
    i_dz, i_dx, i_dy = np.arange(dz), np.arange(dx), np.arange(dy)

    def grid(outer, inner, f):
        a, b = np.meshgrid(outer, inner, indexing="ij")
        return f(a, b).ravel()
    # faces (lulesh-comm.cc:407-510 send, 104-158 receive)
    faces = [
        ("pm", False, True, -T2, np.arange(dx * dy)),
        ("pM", True, False, +T2, dx * dy * (dz - 1) + np.arange(dx * dy)),
        ("rm", False, True, -tp, grid(i_dz, i_dx, lambda i, j: i * dx * dy + j)),
        ("rM", True, False, +tp, grid(i_dz, i_dx, lambda i, j: dx * (dy - 1) + i * dx * dy + j)),
        ("cm", False, True, -1, grid(i_dz, i_dy, lambda i, j: i * dx * dy + j * dx)),
        ("cM", True, False, +1, grid(i_dz, i_dy, lambda i, j: dx - 1 + i * dx * dy + j * dx)),
    ]
    # edges (send 512-725, receive 160-270)
    edges = [
        ("rm cm", False, True, -tp - 1, i_dz * dx * dy),
        ("rm pm", False, True, -T2 - tp, i_dx),
        ("cm pm", False, True, -T2 - 1, i_dy * dx),
        ("rM cM", True, False, tp + 1, dx * dy - 1 + i_dz * dx * dy),
        ("rM pM", True, False, T2 + tp, dx * (dy - 1) + dx * dy * (dz - 1) + i_dx),
        ("cM pM", True, False, T2 + 1, dx * dy * (dz - 1) + dx - 1 + i_dy * dx),
        ("rM cm", True, False, tp - 1, dx * (dy - 1) + i_dz * dx * dy),
        ("rm pM", True, False, T2 - tp, dx * dy * (dz - 1) + i_dx),
        ("cm pM", True, False, T2 - 1, dx * dy * (dz - 1) + i_dy * dx),
        ("rm cM", False, True, -tp + 1, dx - 1 + i_dz * dx * dy),
        ("rM pm", False, True, -T2 + tp, dx * (dy - 1) + i_dx),
        ("cM pm", False, True, -T2 + 1, dx - 1 + i_dy * dx),
    ]
    # corners (send 727-842, receive 272-353)
    corners = [
        ("rm cm pm", False, True, -T2 - tp - 1, [0]),
        ("rm cm pM", True, False, T2 - tp - 1, [dx * dy * (dz - 1)]),
        ("rm cM pm", False, True, -T2 - tp + 1, [dx - 1]),
        ("rm cM pM", True, False, T2 - tp + 1, [dx * dy * (dz - 1) + (dx - 1)]),
        ("rM cm pm", False, True, -T2 + tp - 1, [dx * (dy - 1)]),
        ("rM cm pM", True, False, T2 + tp - 1, [dx * dy * (dz - 1) + dx * (dy - 1)]),
        ("rM cM pm", False, True, -T2 + tp + 1, [dx * dy - 1]),
        ("rM cM pM", True, False, T2 + tp + 1, [dx * dy * dz - 1]),
    ]
    out = []
    for cls, group in ((0, faces), (1, edges), (2, corners)):
        for flags, need_send, need_recv, peer, idx in group:
            out.append((cls, flags.split(), need_send, need_recv, peer,
                        np.asarray(idx, dtype=np.int64)))
    return out


def _kind_args(kind, nx):
    """(dx, dy, dz, doSend, doRecv, planeOnly) of each call site: CalcForceForNodes
    (lulesh.cc:1109-1133), LagrangeLeapFrog (2621-2642), CalcQForElems (1963-1985)."""
    if kind == SBN:
        return nx + 1, nx + 1, nx + 1, True, True, False
    if kind == SYNC_POS_VEL:
        return nx + 1, nx + 1, nx + 1, False, False, False
    return nx, nx, nx, True, True, True


def messages(kind: int, nx: int, tp: int, rank: int, nfields: int, side: str) -> list[dict]:
    """The messages rank sends (side 'send') or receives ('recv'), in order,
    each {peer, count, offset, index}."""
    col, row, plane = location(rank, tp)
    have = {"rm": row != 0, "rM": row != tp - 1, "cm": col != 0, "cM": col != tp - 1,
            "pm": plane != 0, "pM": plane != tp - 1}
    dx, dy, dz, do_send, do_recv, plane_only = _kind_args(kind, nx)
    max_plane = nfields * cache_align((nx + 1) * (nx + 1))   # maxPlaneComm
    max_edge = nfields * cache_align(nx + 1)                  # maxEdgeComm
    counters = [0, 0, 0]
    out = []
    for cls, flags, need_send, need_recv, peer, idx in _table(tp, dx, dy, dz):
        if plane_only and cls > 0:
            continue
        if not all(have[f] for f in flags):
            continue
        if side == "send" and need_send and not do_send:
            continue
        if side == "recv" and need_recv and not do_recv:
            continue
        off = counters[0] * max_plane + counters[1] * max_edge + counters[2] * PAD
        counters[cls] += 1
        out.append({"peer": rank + peer, "count": int(idx.size), "offset": off, "index": idx})
    return out


def buffer_doubles(nx: int, tp: int, rank: int) -> int:
    """SetupCommBuffers' comBufSize (lulesh-init.cc:358-380)."""
    col, row, plane = location(rank, tp)
    rm, rM, cm, cM, pm, pM = (row != 0, row != tp - 1, col != 0, col != tp - 1, plane != 0,
                              plane != tp - 1)
    faces = rm + rM + cm + cM + pm + pM
    edges = ((rm & cm) + (rm & pm) + (cm & pm) + (rM & cM) + (rM & pM) + (cM & pM) +
             (rM & cm) + (rm & pM) + (cm & pM) + (rm & cM) + (rM & pm) + (cM & pm))
    corners = ((rm & cm & pm) + (rm & cm & pM) + (rm & cM & pm) + (rm & cM & pM) +
               (rM & cm & pm) + (rM & cm & pM) + (rM & cM & pm) + (rM & cM & pM))
    return (faces * cache_align((nx + 1) ** 2) * MAX_FIELDS +
            edges * cache_align(nx + 1) * MAX_FIELDS + corners * PAD)


def pack(kind, nx, tp, rank, fields: list[np.ndarray]) -> np.ndarray:
    """CommSend's packing loops: the send buffer of one rank."""
    buf = np.zeros(buffer_doubles(nx, tp, rank))
    for m in messages(kind, nx, tp, rank, len(fields), "send"):
        for fi, f in enumerate(fields):
            o = m["offset"] + fi * m["count"]
            buf[o:o + m["count"]] = f[m["index"]]
    return buf


def unpack(kind, nx, tp, rank, fields: list[np.ndarray], recv: np.ndarray) -> None:
    """CommSBN (lulesh-comm.cc:848-1258: +=, message by message),
    CommSyncPosVel (1261-1681: =) and CommMonoQ (1684-1835: = into the ghost
    elements after numElem, face after face), in place."""
    numElem = nx ** 3
    ghost = numElem
    for m in messages(kind, nx, tp, rank, len(fields), "recv"):
        for fi, f in enumerate(fields):
            o = m["offset"] + fi * m["count"]
            vals = recv[o:o + m["count"]]
            if kind == SBN:
                f[m["index"]] += vals          # one message after another
            elif kind == SYNC_POS_VEL:
                f[m["index"]] = vals
            else:
                f[ghost:ghost + m["count"]] = vals
        if kind == MONOQ:
            ghost += m["count"]


def exchange(kind, nx, tp, fields_by_rank: list[list[np.ndarray]]) -> list[np.ndarray]:
    """Every rank packs, each message travels to its receiver's offset, every
    rank unpacks.  Returns the receive buffers; fields are updated in place."""
    nr = tp ** 3
    nf = len(fields_by_rank[0])
    send = [pack(kind, nx, tp, r, fields_by_rank[r]) for r in range(nr)]
    recv = [np.zeros(buffer_doubles(nx, tp, r)) for r in range(nr)]
    for r in range(nr):
        for m in messages(kind, nx, tp, r, nf, "recv"):
            src = [s for s in messages(kind, nx, tp, m["peer"], nf, "send") if s["peer"] == r]
            assert len(src) == 1 and src[0]["count"] == m["count"]
            n = nf * m["count"]
            recv[r][m["offset"]:m["offset"] + n] = send[m["peer"]][src[0]["offset"]:
                                                                   src[0]["offset"] + n]
    for r in range(nr):
        unpack(kind, nx, tp, r, fields_by_rank[r], recv[r])
    return recv
