"""Calibration harness: force-model parameters fitted to trajectories with a
PyTorch optimiser, through the engine's differentiable form.

``TrajectoryLoss.apply(params, sim)`` is a ``torch.autograd.Function``:
forward sets (V0, sigma, k, tau0) of every scenario of ``sim`` from the rows
of ``params`` and runs the episode set up by ``sim.diff_begin``; backward
returns dL/dparams from the engine's hand-written adjoint.  Both run on the
GPU through the C ABI (umans_diff_forward / umans_diff_backward); torch only
carries the parameter tensor and the optimiser.

``windowed_gradient(sim, observed, window)`` is the form to use on long
observations (multiple shooting): the observed horizon is cut into windows
of a few steps, every window starts from the observed state at its start,
and the windows' losses and gradients add up.  A crowd at the calibration
density separates nearby trajectories by ~2.5x per step, so the gradient of
a single 100-step episode leaves the float range; over a window of 10 steps
it stays finite and matches the float64 reference.
"""
from __future__ import annotations

import numpy as np
import torch

__all__ = ["TrajectoryLoss", "calibrate", "windowed_gradient"]


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


def windowed_gradient(sim, observed: dict, window: int = 10, checkpoint_every: int | None = None):
    """Loss and dL/d(V0, sigma, k, tau0) per scenario of ``sim`` over an
    observation cut into windows.

    observed["pos"], ["vel"] (and optionally ["viewdir"]): (T + 1, n, 2)
    states in list order, the state before the first step and after each of
    the T steps.  Window w covers steps [w W, min(T, (w + 1) W)); it starts
    from the observed state at its first step and is compared with the
    observed positions after each of its steps.  The loss is
    1 / (T n_s) sum_t sum_i |p_i(t) - observed_i(t)|^2 per scenario s of n_s
    agents (the mean squared error over the horizon when the scenarios have
    equal agent counts), summed over the scenarios.  The simulation is left
    at the last window's start state.  Returns (loss, grad[num_scenarios, 4]).
    """
    pos = np.asarray(observed["pos"], np.float32)
    vel = np.asarray(observed["vel"], np.float32)
    view = observed.get("viewdir")
    T = pos.shape[0] - 1
    if T < 1 or pos.shape[1:] != (sim.n, 2) or vel.shape != pos.shape:
        raise ValueError("observed states must have shape (T + 1, n, 2) with T >= 1")
    if window < 1:
        raise ValueError("window must be at least one step")
    counts = np.diff(np.asarray(sim.offsets)) if hasattr(sim, "offsets") else np.array([sim.n])
    if len(set(int(c) for c in counts)) != 1:
        raise ValueError("windowed_gradient needs scenarios of equal agent counts (one loss weight)")
    weight = 1.0 / (T * int(counts[0]))
    loss, grad = 0.0, np.zeros((sim.num_scenarios, 4), np.float64)
    for t0 in range(0, T, window):
        t1 = min(T, t0 + window)
        sim.set_state(pos=pos[t0], vel=vel[t0], viewdir=None if view is None else np.asarray(view[t0], np.float32))
        sim.diff_begin(pos[t0 + 1:t1 + 1], checkpoint_every=checkpoint_every or (t1 - t0), weight=weight)
        loss += sim.diff_forward()
        grad += sim.diff_backward()
    sim.diff_end()
    return loss, grad
