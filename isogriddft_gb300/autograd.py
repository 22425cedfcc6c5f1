"""Differentiable H.Psi (no reference counterpart: the reference has no gradients).

``hpsi(psi, veff, grid_geometry)`` applies H = T + v_eff (trial-fix closure on the
monitor A-grid) through the fused stencil and backpropagates through the same
kernel: the trial-fix kinetic operator is self-adjoint in the cell-volume metric
(W T is symmetric: centred differences with zero ghosts are skew-symmetric and
the folded metric is symmetric), so T^T g = W T (W^-1 g) and
d/dv_eff = sum_o psi_o * g_o.  Other closures are not self-adjoint and raise.
"""

from __future__ import annotations

import torch

from .device import device_grid
from .grid import is_monitor_geometry
from .ops import hpsi_device


class _HPsi(torch.autograd.Function):
    @staticmethod
    def forward(ctx, psi, veff, dg):
        ctx.dg = dg
        ctx.save_for_backward(psi, veff)
        v = veff.reshape(-1).contiguous()
        return hpsi_device(dg, psi.contiguous(), closure="trial_fix", kscale=-0.5, veff=v)

    @staticmethod
    def backward(ctx, g):
        psi, veff = ctx.saved_tensors
        dg = ctx.dg
        w = dg.cell_volumes.to(g.dtype)
        gpsi = gveff = None
        if ctx.needs_input_grad[0]:
            gpsi = hpsi_device(dg, (g / w).contiguous(), closure="trial_fix", kscale=-0.5,
                               veff=veff.reshape(-1).contiguous()) * w
        if ctx.needs_input_grad[1]:
            gveff = (psi * g).sum(0).reshape(veff.shape)
        return gpsi, gveff, None


def hpsi(psi: torch.Tensor, veff: torch.Tensor, grid_geometry) -> torch.Tensor:
    """H psi for a (nb, n) CUDA block, differentiable in psi and veff (n,)."""

    if not is_monitor_geometry(grid_geometry):
        raise NotImplementedError("the differentiable apply covers the trial-fix monitor-grid operator only")
    if psi.dim() != 2 or veff.numel() != psi.shape[1]:
        raise ValueError("psi must be (nb, n) and veff must have n values")
    if psi.dtype != veff.dtype:
        raise ValueError("psi and veff must share a dtype")
    return _HPsi.apply(psi, veff, device_grid(grid_geometry))
