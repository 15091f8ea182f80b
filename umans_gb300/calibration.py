"""Calibration harness: force-model parameters fitted to trajectories with a
PyTorch optimiser, through the engine's differentiable form.

``TrajectoryLoss.apply(params, sim)`` is a ``torch.autograd.Function``:
forward sets (V0, sigma, k, tau0) of every scenario of ``sim`` from the rows
of ``params`` and runs the episode set up by ``sim.diff_begin``; backward
returns dL/dparams from the engine's hand-written adjoint.  Both run on the
GPU through the C ABI (umans_diff_forward / umans_diff_backward); torch only
carries the parameter tensor and the optimiser.
"""
from __future__ import annotations

import numpy as np
import torch

__all__ = ["TrajectoryLoss", "calibrate"]


class TrajectoryLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params: torch.Tensor, sim) -> torch.Tensor:
        p = params.detach().to("cpu", torch.float32).numpy().reshape(-1, 4)
        if p.shape[0] != sim.num_scenarios:
            raise ValueError("params needs one row of (V0, sigma, k, tau0) per scenario")
        for k in range(p.shape[0]):
            sim.set_force_params(p[k], k)
        ctx.sim = sim
        ctx.shape, ctx.dtype, ctx.device = params.shape, params.dtype, params.device
        return torch.tensor(sim.diff_forward(), dtype=torch.float64)

    @staticmethod
    def backward(ctx, grad_out):
        d = ctx.sim.diff_backward()
        g = torch.from_numpy(np.ascontiguousarray(d)).to(ctx.device, ctx.dtype).reshape(ctx.shape)
        return g * grad_out.to(ctx.device, ctx.dtype), None


def calibrate(sim, params0, iterations: int = 20, lr: float = 0.05):
    """Adam on (V0, sigma, k, tau0) per scenario; returns (params, losses)."""
    p = torch.tensor(np.asarray(params0, np.float32).reshape(-1, 4), requires_grad=True)
    opt = torch.optim.Adam([p], lr=lr)
    losses = []
    for _ in range(iterations):
        opt.zero_grad()
        loss = TrajectoryLoss.apply(p, sim)
        loss.backward()
        opt.step()
        with torch.no_grad():
            p.clamp_(min=1e-3)
        losses.append(float(loss))
    return p.detach().numpy(), losses
