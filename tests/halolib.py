"""Helpers of the halo tests: random per-rank fields, the message transport
between ranks' buffers, and a CPU application of a plan's value lists (to
check a plan without a GPU)."""
import numpy as np

# fields each call site exchanges (lulesh.cc:1109-1133, 2621-2642, 1963-1985,
# 2723-2729): (kind, nfields)
CALL_SITES = {"forces": ("sbn", 3), "pos_vel": ("sync_pos_vel", 6), "monoq": ("monoq", 3),
              "nodal_mass": ("sbn", 1)}
KIND_ID = {"sbn": 0, "sync_pos_vel": 1, "monoq": 2}


def field_length(kind: str, nx: int) -> int:
    if kind == "monoq":
        return nx ** 3 + 6 * nx * nx  # numElem + every possible ghost (lulesh.cc:1955-1958)
    return (nx + 1) ** 3


def random_fields(kind: str, nx: int, tp: int, nfields: int, seed: int):
    rng = np.random.default_rng(seed)
    n = field_length(kind, nx)
    return [[rng.standard_normal(n) for _ in range(nfields)] for _ in range(tp ** 3)]


def transport(send_msgs, recv_msgs, send_bufs, recv_bufs, nfields: int) -> None:
    """Copy every message from its sender's send buffer to its receiver's
    receive buffer: message m of rank r's receive list comes from the one
    message of the peer's send list addressed to r."""
    for r, msgs in enumerate(recv_msgs):
        for m in msgs:
            src = [s for s in send_msgs[m["peer"]] if s["peer"] == r]
            assert len(src) == 1 and src[0]["count"] == m["count"], (r, m)
            n = nfields * m["count"]
            recv_bufs[r][m["offset"]:m["offset"] + n] = \
                send_bufs[m["peer"]][src[0]["offset"]:src[0]["offset"] + n]


def cpu_pack(entries: dict, fields, buf) -> None:
    idx, pos, stride = entries["index"], entries["bufpos"], entries["stride"]
    for f, a in enumerate(fields):
        buf[pos + f * stride] = a[idx]


def cpu_unpack(kind: str, entries: dict, fields, buf) -> None:
    idx, pos, stride = entries["index"], entries["bufpos"], entries["stride"]
    for f, a in enumerate(fields):
        vals = buf[pos + f * stride]
        for t, v in zip(idx, vals):       # in the plan's application order
            a[t] = a[t] + v if kind == "sbn" else v
