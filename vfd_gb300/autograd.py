"""torch.autograd wrapper of the step's adjoint (vfd_adjoint_forward / _backward).

    x_T, v_T = rollout(sim, x0, v0, viscosity, boundary_viscosity, steps=60, checkpoint_every=10)
    loss = ((x_T - target) ** 2).sum(1).mean()
    loss.backward()          # gradients in x0.grad, v0.grad, viscosity.grad, boundary_viscosity.grad

The rollout restarts `sim` from (x0, v0) with the given viscosities (SetDescription +
SetFluidObjects, as a fresh run of the reference would), runs `steps` steps on the GPU
and returns the final positions and velocities. The backward pass is the library's
hand-written adjoint; torch only carries tensors across the boundary (host copies, as
the C-ABI takes host arrays).
"""
from __future__ import annotations

import numpy as np
import torch


def _restart(sim, x0, v0, viscosity: float, boundary_viscosity: float):
    desc = sim.GetDescription()
    desc["Viscosity"] = float(viscosity)
    desc["BoundaryViscosity"] = float(boundary_viscosity)
    sim.SetDescription(desc)
    sim.SetFluidObjects(np.asarray(x0, np.float32), np.asarray(v0, np.float32))


class DFSPHRollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x0, v0, viscosity, boundary_viscosity, sim, steps, checkpoint_every):
        _restart(sim, x0.detach().cpu().numpy(), v0.detach().cpu().numpy(), float(viscosity), float(boundary_viscosity))
        sim.AdjointForward(steps, checkpoint_every)
        x, v, _ = sim.GetState()
        ctx.sim = sim
        ctx.dev = x0.device
        return torch.from_numpy(x).to(x0.device), torch.from_numpy(v).to(x0.device)

    @staticmethod
    def backward(ctx, x_bar, v_bar):
        xb = (x_bar if x_bar is not None else torch.zeros(1)).detach().cpu().float().numpy()
        vb = (v_bar if v_bar is not None else torch.zeros(1)).detach().cpu().float().numpy()
        n = ctx.sim.GetParticleCount()
        if x_bar is None:
            xb = np.zeros((n, 3), np.float32)
        if v_bar is None:
            vb = np.zeros((n, 3), np.float32)
        x0b, v0b, pb = ctx.sim.AdjointBackward(xb, vb)
        t = lambda a: torch.from_numpy(np.asarray(a)).to(ctx.dev)  # noqa: E731
        return t(x0b), t(v0b), t(pb[0]), t(pb[1]), None, None, None


def rollout(sim, x0, v0, viscosity, boundary_viscosity, steps: int, checkpoint_every: int = 10):
    """Differentiable `steps`-step run of `sim` from (x0, v0); see the module docstring."""
    vis = viscosity if torch.is_tensor(viscosity) else torch.tensor(float(viscosity))
    bvis = boundary_viscosity if torch.is_tensor(boundary_viscosity) else torch.tensor(float(boundary_viscosity))
    return DFSPHRollout.apply(x0, v0, vis, bvis, sim, steps, checkpoint_every)
