"""Field comparison used by the parity tests.

Relative error of a field is measured elementwise against the oracle value
with an absolute floor proportional to the field's scale:

    err_i = |gpu_i - ref_i| / max(|ref_i|, FLOOR * max_j |ref_j|)

FLOOR = 1e-6: entries more than six orders of magnitude below the field's
largest value (for instance the velocity tail ahead of the Sedov front, or
cut-off values near u_cut) are compared on the field's scale rather than
their own.  The FP64 bar is max_i err_i <= 1e-10.
"""
import numpy as np

FLOOR = 1e-6
FP64_TOL = 1e-10

# delv = vnew - v is a difference of two relative volumes close to 1
# (lulesh.cc:1534); its rounding error is an ulp of the relative volume, so
# it is measured on that scale: the denominator of entry i is
# max(|delv_i|, |vnew_i|).
DIFFERENCE_FIELDS = {"delv": "vnew"}


def field_rel_err(gpu: np.ndarray, ref: np.ndarray, floor: float = FLOOR) -> float:
    gpu = np.asarray(gpu, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    if gpu.shape != ref.shape:
        raise ValueError("shape mismatch")
    scale = float(np.max(np.abs(ref))) if ref.size else 0.0
    if scale == 0.0:
        return float(np.max(np.abs(gpu))) if gpu.size else 0.0
    den = np.maximum(np.abs(ref), floor * scale)
    return float(np.max(np.abs(gpu - ref) / den))


def diff_field_rel_err(gpu: np.ndarray, ref: np.ndarray, operand: np.ndarray) -> float:
    gpu = np.asarray(gpu, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    den = np.maximum(np.abs(ref), np.abs(np.asarray(operand, dtype=np.float64)))
    den = np.where(den == 0.0, 1.0, den)
    return float(np.max(np.abs(gpu - ref) / den)) if ref.size else 0.0


def compare_states(gpu: dict, ref: dict, fields) -> dict:
    out = {}
    for f in fields:
        if f in DIFFERENCE_FIELDS and DIFFERENCE_FIELDS[f] in ref:
            out[f] = diff_field_rel_err(gpu[f], ref[f], ref[DIFFERENCE_FIELDS[f]])
        else:
            out[f] = field_rel_err(gpu[f], ref[f])
    return out


def normwise_rel_err(gpu: np.ndarray, ref: np.ndarray) -> float:
    """max_i |gpu_i - ref_i| / max_i |ref_i|"""
    scale = float(np.max(np.abs(ref))) if np.size(ref) else 0.0
    d = float(np.max(np.abs(np.asarray(gpu) - np.asarray(ref)))) if np.size(ref) else 0.0
    return d / scale if scale else d


def symmetry_deltas(e: np.ndarray, nx: int) -> dict:
    """Plane-0 symmetry deltas of the energy field, as the reference's
    end-of-run self-check computes them (lulesh-util.cc:197-212): over
    j < k < nx, |e[j*nx+k] - e[k*nx+j]|, its maximum and sum, and the largest
    difference relative to e[k*nx+j]."""
    j, k = np.triu_indices(nx, 1)
    a, b = e[j * nx + k], e[k * nx + j]
    d = np.abs(a - b)
    with np.errstate(divide="ignore", invalid="ignore"):
        rel = np.where(d > 0, d / b, 0.0)
    return {"MaxAbsDiff": float(d.max(initial=0.0)), "TotalAbsDiff": float(d.sum()),
            "MaxRelDiff": float(np.nanmax(rel, initial=0.0))}


def total_energy(state: dict) -> float:
    """Internal sum(e * volo) plus kinetic sum(m |u|^2) / 2 of a state dict
    holding e, volo, nodalMass, xd, yd, zd."""
    ke = 0.5 * np.sum(state["nodalMass"] * (state["xd"] ** 2 + state["yd"] ** 2 +
                                            state["zd"] ** 2))
    return float(np.sum(state["e"] * state["volo"]) + ke)
