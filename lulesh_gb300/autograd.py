"""The leap-frog path as torch.autograd.Functions.

Thin bindings over the C ABI's adjoint:
  TerminalEnergy    J(e0, hgcoef), the total internal energy sum(e * volo) of a
                    fixed set of elements after a fixed number of cycles with a
                    frozen time-step sequence, from the initial energy field
                    e0; the forward also computes the gradients (lg_adjoint);
  FinalEnergyField  the final energy field e(e0, hgcoef) itself, so that any
                    torch loss of it backpropagates (lg_adjoint_vjp).
Tensors live on the host; the GPU work happens inside the library.
"""
from __future__ import annotations

import numpy as np
import torch

from . import Domain


class TerminalEnergyProblem:
    """A Sedov problem, a cycle count, a frozen dt sequence and an element mask.

    The dt sequence and the mask come from one forward run of `e_base`
    (the mask: element centroids within `radius` of the origin at the end),
    unless given (`dts`: ncycles steps; `mask`: numElem booleans)."""

    def __init__(self, nx: int = 48, numReg: int = 11, ncycles: int = 200, ckpt: int = 20,
                 e_base: np.ndarray | None = None, radius: float = 0.5,
                 precision: str = "fp64", device: int = 0, dts: np.ndarray | None = None,
                 mask: np.ndarray | None = None):
        self.nx, self.ncycles, self.ckpt = nx, ncycles, ckpt
        self.dom = Domain(nx, numReg, its=10 ** 9, precision=precision, device=device)
        self.e_init = self.dom.field("e")
        self.e_base = self.e_init.copy() if e_base is None else np.asarray(e_base, np.float64)
        self.hg_base = self.dom.scalar("hgcoef")
        if dts is None or mask is None:
            self.dom.set_field("e", self.e_base)
            self.dom.dt_record(ncycles)
            if self.dom.step(ncycles) != 0:
                raise RuntimeError("forward run failed")
            rec_dts = self.dom.dt_get(ncycles)
            rec_mask = centroid_mask(self.dom, radius)
            self.dom.dt_record(0)
        self.dts = np.asarray(dts, np.float64) if dts is not None else rec_dts
        self.mask = np.asarray(mask, bool) if mask is not None else rec_mask
        if self.dts.size != ncycles or self.mask.size != self.e_init.size:
            raise ValueError("dts must hold ncycles steps and mask one flag per element")
        self.dom.dt_freeze(self.dts)

    def objective(self, e0: np.ndarray, hgcoef: float) -> float:
        """J with the frozen steps, forward only (lg_step)."""
        d = self.dom
        d.reset()
        d.set_field("e", e0)
        d.set_scalar("hgcoef", hgcoef)
        if d.step(self.ncycles) != 0:
            raise RuntimeError("forward run failed")
        return float(np.sum(d.field("e")[self.mask] * d.field("volo")[self.mask]))

    def value_and_grad(self, e0: np.ndarray, hgcoef: float):
        d = self.dom
        d.reset()
        d.set_field("e", e0)
        d.set_scalar("hgcoef", hgcoef)
        return d.adjoint(self.ncycles, self.mask, self.ckpt)

    def final_field(self, e0: np.ndarray, hgcoef: float, name: str = "e") -> np.ndarray:
        """A field of the final state after the frozen-step cycles from e0."""
        d = self.dom
        d.reset()
        d.set_field("e", e0)
        d.set_scalar("hgcoef", hgcoef)
        if d.step(self.ncycles) != 0:
            raise RuntimeError("forward run failed")
        return d.field(name)

    def vjp(self, e0: np.ndarray, hgcoef: float, seeds: dict, want=("e",)):
        """dJ/d(initial fields in `want`) and dJ/dhgcoef for an objective J of
        the final state whose gradient is `seeds` (lg_adjoint_vjp)."""
        d = self.dom
        d.reset()
        d.set_field("e", e0)
        d.set_scalar("hgcoef", hgcoef)
        return d.adjoint_vjp(self.ncycles, seeds, want, self.ckpt)


def centroid_mask(dom: Domain, radius: float) -> np.ndarray:
    nl = dom.field("nodelist").reshape(-1, 8)
    c = np.stack([dom.field(f)[nl].mean(axis=1) for f in ("x", "y", "z")], axis=1)
    return np.sqrt(np.sum(c * c, axis=1)) < radius


class TerminalEnergy(torch.autograd.Function):
    """J(e0, hgcoef) for a TerminalEnergyProblem; differentiable in both."""

    @staticmethod
    def forward(ctx, e0: torch.Tensor, hgcoef: torch.Tensor, problem: TerminalEnergyProblem):
        J, ge, gh = problem.value_and_grad(e0.detach().cpu().double().numpy(), float(hgcoef))
        ctx.save_for_backward(torch.from_numpy(ge), torch.tensor(gh, dtype=torch.float64))
        return torch.tensor(J, dtype=torch.float64)

    @staticmethod
    def backward(ctx, gJ):
        ge, gh = ctx.saved_tensors
        return gJ * ge, gJ * gh, None


class FinalEnergyField(torch.autograd.Function):
    """The final energy field e(e0, hgcoef) of a TerminalEnergyProblem's
    cycles, differentiable in both: any torch loss of the final field
    backpropagates through lg_adjoint_vjp."""

    @staticmethod
    def forward(ctx, e0: torch.Tensor, hgcoef: torch.Tensor, problem: TerminalEnergyProblem):
        e0n = e0.detach().cpu().double().numpy().copy()
        ctx.problem, ctx.e0, ctx.hg = problem, e0n, float(hgcoef)
        return torch.from_numpy(problem.final_field(e0n, float(hgcoef)).copy())

    @staticmethod
    def backward(ctx, g):
        seed = g.detach().cpu().double().numpy()
        grads, gh = ctx.problem.vjp(ctx.e0, ctx.hg, {"e": seed}, want=("e",))
        return torch.from_numpy(grads["e"]), torch.tensor(gh, dtype=torch.float64), None
