"""Differentiable projection loss for PyTorch over the C ABI.

``ProjectionLoss`` evaluates, on the GPU, the loss

    J = sum over cut cells of p * (-nz) * WlLh      (pressure force on the
        solid, the Clpz1 sum of PrintDragLiftCoef, Solver.f90:684-706)
      + 1/2 ||D u||^2                                 (divergence of the
        corrected velocity, ComputePUVW.f90:181-232)

of one pressure projection, and its gradient with respect to the predicted
velocity (u*, v*, w*) and a per-cell density field by the hand-written
adjoint (one more solve with the same operator).  ``projection_loss`` wraps
it in a ``torch.autograd.Function``.

Fields are float64 CPU tensors of shape (K+2, J+2, I+2): the memory layout of
the Fortran arrays (I+2, J+2, K+2).
"""
from __future__ import annotations

import numpy as np
import torch

from . import workloads as W
from .projection import Projection


def _to_np(t: torch.Tensor) -> np.ndarray:
    if t.dtype != torch.float64 or t.device.type != "cpu":
        raise ValueError("a CPU float64 tensor is required")
    return np.asfortranarray(t.detach().contiguous().numpy().T)


def _to_t(a: np.ndarray) -> torch.Tensor:
    return torch.from_numpy(np.ascontiguousarray(a.T))


class ProjectionLoss:
    """Loss and adjoint gradient of one projection on a fixed geometry."""

    def __init__(self, workload, g=None, rel_tol=1e-12, adjoint_rel_tol=1e-10, **opts):
        """``rel_tol``: tolerance of the pressure solve; ``adjoint_rel_tol``:
        tolerance of the adjoint solve, whose right-hand side (the weights g,
        concentrated on the cut cells) puts its FP64 rounding floor near
        1e-11 at 128^3."""
        self.w = workload
        self.g = W.pressure_force_weights(workload) if g is None else np.asfortranarray(g)
        self.rel_tol, self.adjoint_rel_tol = rel_tol, adjoint_rel_tol
        self.proj = Projection.for_workload(workload, rel_tol=rel_tol, **opts)

    def forward(self, u, v, w, rho=None):
        J0, J1, st = self.proj.loss_forward(self.w, self.g, rho=rho, pred=(u, v, w))
        return J0 + J1, (J0, J1), st

    def backward(self):
        self.proj.set_opts(rel_tol=self.adjoint_rel_tol)
        try:
            grads, st = self.proj.loss_backward(self.w.shape_g)
        finally:
            self.proj.set_opts(rel_tol=self.rel_tol)
        return grads, st


class _Fn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u, v, w, rho, runner):
        J, parts, _ = runner.forward(_to_np(u), _to_np(v), _to_np(w), _to_np(rho))
        (gu, gv, gw, grho), _ = runner.backward()
        ctx.save_for_backward(_to_t(gu), _to_t(gv), _to_t(gw), _to_t(grho))
        return torch.tensor(J, dtype=torch.float64)

    @staticmethod
    def backward(ctx, gJ):
        gu, gv, gw, grho = ctx.saved_tensors
        return gJ * gu, gJ * gv, gJ * gw, gJ * grho, None


def projection_loss(u: torch.Tensor, v: torch.Tensor, w: torch.Tensor, rho: torch.Tensor,
                    runner: ProjectionLoss) -> torch.Tensor:
    """J(u*, v*, w*, rho) with gradients through the hand-written adjoint."""
    return _Fn.apply(u, v, w, rho, runner)
