"""The differentiable-wall objective and its central differences on the f64
oracle - test infrastructure: the reference an adjoint's gradient is checked
against.

Objective: the mean displacement |p_i(T) - p_i(0)| of the 256 bricks of
scene.brick_wall_c5 after T steps. Parameters theta: the sphere's initial
velocity (3), the bricks' friction mu, and the penalty cap penalty_max (the
hard bonds' stand-in for a stiffness). Central differences use an absolute
step h for the velocity and mu, and a step relative to the value for the
penalty cap.
"""
from __future__ import annotations

import importlib

import numpy as np

from oracle import Oracle, TangentOracle

NAMES = ("v0_x", "v0_y", "v0_z", "mu", "penalty_max")
STEPS = 30  # the horizon whose differences converge (over 60 steps contact events flip within +-h)
H = (1e-4, 5e-5)


def theta0(abi) -> np.ndarray:
    return np.array([0.0, 8.0, 0.0, 0.6, abi.default_params().penalty_max])


def params_of(abi, s, theta, order):
    """The wall's parameters at theta; `order` is the primal sweep's body
    order: None for the reference engine's (newest body first), or
    abi.ORDER_PRIORITY for the colour order of the integer-priority
    colouring (the CUDA backend's schedule)."""
    kw = {} if order is None else {"body_order": order}
    return abi.default_params(**s.params, penalty_max=float(theta[4]), **kw)


def objective(abi, scenes, theta, steps: int, order=None) -> float:
    s = scenes.brick_wall_c5(mu=float(theta[3]), sphere_velocity=tuple(float(v) for v in theta[:3]))
    params = params_of(abi, s, theta, order)
    w = s.world()
    o = Oracle(params, w)
    o.step(steps)
    b0, b1 = s.meta["bricks"]
    return float(np.linalg.norm(o.state().pos[b0:b1] - w.pos[b0:b1], axis=1).mean())


def seeds(abi, s, w):
    """The seeds of the gradient's five directions, as (kind, index, comp,
    direction): the sphere's velocity components (0-2), every brick's
    friction (3), the penalty cap (4)."""
    sphere = w.n_bodies - 1
    b0, b1 = s.meta["bricks"]
    out = [(abi.SEED_VELOCITY, sphere, k, k) for k in range(3)]
    out += [(abi.SEED_FRICTION, b, 0, 3) for b in range(b0, b1)]
    out.append((abi.SEED_PENALTY_MAX, 0, 0, 4))
    return out


def gradient_from_tangents(s, w, pos, tan, theta):
    """The objective and its gradient from the positions after the run and
    their derivatives along the five directions."""
    b0, b1 = s.meta["bricks"]
    d = pos[b0:b1] - w.pos[b0:b1]
    dist = np.linalg.norm(d, axis=1)
    grad = np.einsum("ij,ijk->k", d / dist[:, None], tan[b0:b1]) / (b1 - b0)
    grad[4] *= theta[4]  # per relative change of the cap, as the differences step it
    return float(dist.mean()), grad


def upstream(s, w, pos):
    """dL/dpos of the objective at positions `pos` (n x 3): the upstream
    gradient a backward pass contracts with the position derivatives."""
    b0, b1 = s.meta["bricks"]
    g = np.zeros_like(pos)
    d = pos[b0:b1] - w.pos[b0:b1]
    g[b0:b1] = d / np.linalg.norm(d, axis=1)[:, None] / (b1 - b0)
    return g


def tangent_gradient(abi, scenes, theta, steps: int, order=None):
    """The objective and its exact derivative along theta, from the tangent
    oracle: the sphere's velocity components, every brick's friction and the
    penalty cap each carry one direction."""
    s = scenes.brick_wall_c5(mu=float(theta[3]), sphere_velocity=tuple(float(v) for v in theta[:3]))
    params = params_of(abi, s, theta, order)
    w = s.world()
    o = TangentOracle(params, w)
    for kind, index, comp, direction in seeds(abi, s, w):
        if kind == abi.SEED_VELOCITY:
            o.seed_velocity(index, comp, direction)
        elif kind == abi.SEED_FRICTION:
            o.seed_friction(index, direction)
        else:
            o.seed_penalty_max(direction)
    o.step(steps)
    pos, tan = o.positions()
    return gradient_from_tangents(s, w, pos, tan, theta)


def central_differences(abi, scenes, theta, steps: int, h: float, order=None) -> np.ndarray:
    scale = np.array([1.0, 1.0, 1.0, 1.0, theta[4]])
    g = np.zeros(len(theta))
    for i in range(len(theta)):
        e = np.zeros(len(theta))
        e[i] = h * scale[i]
        g[i] = (objective(abi, scenes, theta + e, steps, order) - objective(abi, scenes, theta - e, steps, order)) / (2 * h)
    return g


def modules():
    return importlib.import_module("avbd-sandbox_gb300.abi"), importlib.import_module("avbd-sandbox_gb300.scene")
