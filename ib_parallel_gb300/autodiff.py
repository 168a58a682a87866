"""torch.autograd binding of the library's discrete adjoint (ib_adjoint_forward / _backward).

``FrameForces.apply(frames, sim, K)`` advances ``sim`` (stationary rigid bodies, num_stat) by
``len(frames)`` steps with the moving frame's (u, v, W) of each step and returns the force
coefficients (nsteps, nbody, 2); its backward runs the library's reverse sweep (checkpoints every
K steps, segments recomputed) and returns dJ/dframes.  Frames built with torch operations from
kinematic parameters (pitching amplitude, frequency, phase) carry the gradient on to them.
"""
from __future__ import annotations

import math

import torch


class FrameForces(torch.autograd.Function):
    @staticmethod
    def forward(ctx, frames: torch.Tensor, sim, K: int = 20):
        fr = frames.detach().to("cpu", torch.float64).numpy()
        forces = sim.adjoint_forward(fr, K)
        ctx.sim = sim
        return torch.from_numpy(forces.copy()).to(frames.device)

    @staticmethod
    def backward(ctx, grad_forces: torch.Tensor):
        g = grad_forces.detach().to("cpu", torch.float64).contiguous().numpy()
        dframes = ctx.sim.adjoint_backward(g)
        return torch.from_numpy(dframes).to(grad_forces.device), None, None


def pitching_frames(nsteps: int, dt: float, amplitude, frequency, phase, speed: float = 1.0) -> torch.Tensor:
    """The frame of a body pitching about the frame's centre in a stream of the given speed, seen
    from the body: the stream reaches it at incidence alpha(t) = A sin(2 pi f t + phi) (the body
    turns clockwise by alpha), so the grid moves at -U (cos alpha, sin alpha) and turns at
    -dalpha/dt.  Step n uses the motion at t = (n + 1) dt.  A, f, phi may be tensors that require
    grad."""
    t = dt * torch.arange(1, nsteps + 1, dtype=torch.float64)
    arg = 2.0 * math.pi * frequency * t + phase
    alpha = amplitude * torch.sin(arg)
    alpha_dot = amplitude * 2.0 * math.pi * frequency * torch.cos(arg)
    u = -speed * torch.cos(alpha)
    v = -speed * torch.sin(alpha)
    return torch.stack([u, v, -alpha_dot], dim=1)


def lift_drag(forces: torch.Tensor, frames: torch.Tensor, speed: float = 1.0):
    """Per-step lift and drag coefficients of body 0 in the stream's axes, from the body-frame
    force coefficients and the frame (the stream direction is -(u, v) / |(u, v)|)."""
    u, v = frames[:, 0], frames[:, 1]
    nrm = torch.sqrt(u * u + v * v)
    ex, ey = -u / nrm, -v / nrm
    cx, cy = forces[:, 0, 0], forces[:, 0, 1]
    drag = cx * ex + cy * ey
    lift = -cx * ey + cy * ex
    return lift, drag


__all__ = ["FrameForces", "pitching_frames", "lift_drag"]
