"""The adjoint study's inputs, shared by the GPU tests and the golden-fixture
script: the Sedov problem at s=48 with 11 regions, 200 cycles; the initial
energy field is the reference set-up plus N(0, 1e-3 * e0) noise on the 1,000
elements nearest the origin (e0 = the deposited origin energy, seed 2024);
16 seeded directions supported on those elements (seed 7).  Relative step
1e-6: a perturbation of the energy field has 2-norm 1e-6 times the 2-norm of
the field over the perturbed elements; hgcoef moves by 1e-6 * hgcoef."""
import numpy as np

NX, NREG, NCYCLES, CKPT = 48, 11, 200, 20
NNOISE, NDIR, REL_STEP = 1000, 16, 1e-6


def nearest_elements(nx: int, n: int) -> np.ndarray:
    h = 1.125 / nx
    k, j, i = np.meshgrid(np.arange(nx), np.arange(nx), np.arange(nx), indexing="ij")
    r2 = ((i + 0.5) * h) ** 2 + ((j + 0.5) * h) ** 2 + ((k + 0.5) * h) ** 2
    order = np.lexsort((np.arange(nx ** 3), r2.ravel()))
    return order[:n]


def initial_energy(e_setup: np.ndarray, nx: int = NX, nnoise: int = NNOISE):
    """(noisy initial field, indices of the noisy elements)"""
    idx = nearest_elements(nx, min(nnoise, nx ** 3))
    e0 = float(e_setup[0])
    rng = np.random.default_rng(2024)
    e = e_setup.copy()
    e[idx] += rng.normal(0.0, 1e-3 * e0, idx.size)
    return e, idx


def directions(idx: np.ndarray, e: np.ndarray, ndir: int = NDIR) -> np.ndarray:
    """ndir perturbations of the energy field supported on idx, each with
    2-norm REL_STEP * |e[idx]|"""
    rng = np.random.default_rng(7)
    out = np.zeros((ndir, e.size))
    scale = REL_STEP * np.linalg.norm(e[idx])
    for r in range(ndir):
        d = rng.standard_normal(idx.size)
        out[r, idx] = d / np.linalg.norm(d) * scale
    return out
