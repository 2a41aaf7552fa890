"""torch.autograd.Function over the differentiable step of the C ABI.

`StepFunction.apply(theta, backend, build, steps)` runs `steps` steps of the
world that `build(theta)` describes through `avbd_adjoint_forward` and
returns the body positions after them (n x 3, float64). Its backward is
`avbd_adjoint_backward`: the vector-Jacobian product of those positions with
the upstream gradient, one entry per component of theta. Component d of
theta is direction d of the device's tangents: `build` returns the world at
theta and the seeds (abi.SEED_*) that tie each of its inputs to a direction,
so at most abi.TANGENT_DIMS parameters.

    def build(th):                    # th: numpy float64, the current theta
        s = scene.brick_wall_c5(mu=th[3], sphere_velocity=th[:3])
        w = s.world()
        seeds = [(abi.SEED_VELOCITY, w.n_bodies - 1, k, k) for k in range(3)]
        seeds += [(abi.SEED_FRICTION, b, 0, 3) for b in range(1, 257)]
        return w, seeds

    theta = torch.tensor([0, 8, 0, 0.6], dtype=torch.float64, requires_grad=True)
    pos = StepFunction.apply(theta, gpu, build, 30)
    loss = (pos[1:257] - pos0[1:257]).norm(dim=1).mean()
    loss.backward()                   # theta.grad = dloss/dtheta

The backend holds one differentiable run at a time: a forward on the same
GpuBackend replaces the previous run, so the backward of a forward must come
before the next forward on that backend (a stale backward raises).
The positions come back on theta's device; the gradient follows them.
"""
from __future__ import annotations

import numpy as np

from . import abi


def _torch():
    import torch

    return torch


class _Run:
    """Which forward a GpuBackend's differentiable state belongs to."""

    counter = 0


def _make_function():
    torch = _torch()

    class StepFunction(torch.autograd.Function):
        @staticmethod
        def forward(ctx, theta, backend, build, steps):
            th = theta.detach().to("cpu", torch.float64).numpy().copy()
            if th.ndim != 1 or th.size > abi.TANGENT_DIMS:
                raise ValueError(f"theta must be a vector of at most {abi.TANGENT_DIMS} parameters")
            world, seeds = build(th)
            for kind, index, comp, d in seeds:
                if not 0 <= d < th.size:
                    raise ValueError(f"seed direction {d} has no component of theta (size {th.size})")
            backend.adjoint_forward(world, int(steps), seeds)
            pos, _, _ = backend.adjoint_read()
            _Run.counter += 1
            backend._autograd_run = _Run.counter
            ctx.run = _Run.counter
            ctx.backend = backend
            ctx.size = th.size
            return torch.from_numpy(pos).to(theta.device)

        @staticmethod
        def backward(ctx, grad_pos):
            be = ctx.backend
            if getattr(be, "_autograd_run", None) != ctx.run:
                raise RuntimeError("StepFunction.backward: the backend ran another differentiable forward since "
                                   "this one; call backward before the next forward on the same GpuBackend")
            g = grad_pos.detach().to("cpu", torch.float64).contiguous().numpy()
            grad = be.adjoint_backward(np.ascontiguousarray(g))
            return torch.from_numpy(grad[:ctx.size].copy()).to(grad_pos.device), None, None, None

    return StepFunction


_FN = None


def step_function():
    """The torch.autograd.Function class (built on first use so that importing
    this module does not import torch)."""
    global _FN
    if _FN is None:
        _FN = _make_function()
    return _FN


def __getattr__(name):
    if name == "StepFunction":
        return step_function()
    raise AttributeError(name)
