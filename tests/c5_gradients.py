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


def objective(abi, scenes, theta, steps: int) -> float:
    s = scenes.brick_wall_c5(mu=float(theta[3]), sphere_velocity=tuple(float(v) for v in theta[:3]))
    params = abi.default_params(**s.params, penalty_max=float(theta[4]))
    w = s.world()
    o = Oracle(params, w)
    o.step(steps)
    b0, b1 = s.meta["bricks"]
    return float(np.linalg.norm(o.state().pos[b0:b1] - w.pos[b0:b1], axis=1).mean())


def tangent_gradient(abi, scenes, theta, steps: int):
    """The objective and its exact derivative along theta, from the tangent
    oracle: the sphere's velocity components, every brick's friction and the
    penalty cap each carry one direction."""
    s = scenes.brick_wall_c5(mu=float(theta[3]), sphere_velocity=tuple(float(v) for v in theta[:3]))
    params = abi.default_params(**s.params, penalty_max=float(theta[4]))
    w = s.world()
    o = TangentOracle(params, w)
    sphere = w.n_bodies - 1
    b0, b1 = s.meta["bricks"]
    for k in range(3):
        o.seed_velocity(sphere, k, k)
    for b in range(b0, b1):
        o.seed_friction(b, 3)
    o.seed_penalty_max(4)
    o.step(steps)
    pos, tan = o.positions()
    d = pos[b0:b1] - w.pos[b0:b1]
    dist = np.linalg.norm(d, axis=1)
    grad = np.einsum("ij,ijk->k", d / dist[:, None], tan[b0:b1]) / (b1 - b0)
    grad[4] *= theta[4]  # per relative change of the cap, as the differences step it
    return float(dist.mean()), grad


def central_differences(abi, scenes, theta, steps: int, h: float) -> np.ndarray:
    scale = np.array([1.0, 1.0, 1.0, 1.0, theta[4]])
    g = np.zeros(len(theta))
    for i in range(len(theta)):
        e = np.zeros(len(theta))
        e[i] = h * scale[i]
        g[i] = (objective(abi, scenes, theta + e, steps) - objective(abi, scenes, theta - e, steps)) / (2 * h)
    return g


def modules():
    return importlib.import_module("avbd-sandbox_gb300.abi"), importlib.import_module("avbd-sandbox_gb300.scene")
