"""The differentiable step on the device (avbd_adjoint_forward / _read /
_backward, through the C ABI) against the tangent oracle.

The device's differentiable step runs the f64 engine's operations on a dual
scalar (values in f64, five directional derivatives), visiting bodies in the
colour order of the integer-priority colouring; the tangent oracle does the
same on the CPU with AVBD_ORDER_PRIORITY. So the values must agree to f64
rounding and the derivatives to a relative 1e-7 of their largest component
(the same operations; only the dual arithmetic's own rounding differs where
the compilers order a product's terms differently).

The differentiable wall (C5): the device's gradient of the mean brick
displacement after 30 steps, taken with the backward (vector-Jacobian
product) and from the read tangents, equals the tangent oracle's exact
gradient (tests/golden/c5_gradients_priority.json) within 2e-4 relative and,
along the sphere's y velocity, the oracle's central differences within 5 %.
On the wall the device's values equal the tangent oracle's bit for bit
through step 7; from step 8 one component differs by an ulp, which the
sphere's impact (from step ~19) amplifies to 1e-9 m at step 25 and 1e-6 m at
step 30, so the wall's bounds are 2e-6 m on positions and 2e-5 of the
largest derivative.
"""
import importlib
import json
import os

import numpy as np
import pytest

import c5_gradients as c5
from oracle import TangentOracle

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "c5_gradients_priority.json")
POS_TOL = 1e-9       # m: f64 values, the same operations
TAN_REL = 1e-7       # of the largest derivative component


@pytest.fixture(scope="module")
def backend_mod():
    return importlib.import_module("avbd-sandbox_gb300.backend")


def run_both(abi, backend_mod, s, steps, seeds, params=None):
    params = params or abi.default_params(**s.params, body_order=abi.ORDER_PRIORITY)
    w = s.world()
    o = TangentOracle(params, w)
    for seed in seeds:
        o.seed(*seed)
    o.step(steps)
    ref = o.positions()
    gpu = backend_mod.GpuBackend(params)
    gpu.adjoint_forward(w, steps, seeds)
    got = gpu.adjoint_read()
    return ref, got, gpu


def check(ref, got, pos_tol=POS_TOL, tan_rel=TAN_REL):
    (opos, otan), (gpos, gtan, gquat) = ref, got
    assert np.all(np.isfinite(gpos)) and np.all(np.isfinite(gtan))
    err = np.max(np.abs(gpos - opos))
    assert err <= pos_tol, err
    scale = max(np.max(np.abs(otan)), 1e-30)
    terr = np.max(np.abs(gtan - otan)) / scale
    assert terr <= tan_rel, terr
    assert np.allclose(np.linalg.norm(gquat, axis=1), 1.0, atol=1e-12)


def generic_seeds(abi, w, nj=0):
    """The last body's velocity (directions 0-2), every body's friction (3),
    the penalty cap (4)."""
    last = w.n_bodies - 1
    seeds = [(abi.SEED_VELOCITY, last, k, k) for k in range(3)]
    seeds += [(abi.SEED_FRICTION, b, 0, 3) for b in range(w.n_bodies)]
    seeds.append((abi.SEED_PENALTY_MAX, 0, 0, 4))
    return seeds


SCENES = {
    "pyramid_small": (lambda sc: sc.pyramid(layers=6), 20),
    "heavy_chain_small": (lambda sc: sc.heavy_chain(links=8, springs=10), 20),
    "breakage": (lambda sc: sc.breakage(), 12),
    "spheres": (lambda sc: sc.spheres_scene(), 20),
    "cube_stack": (lambda sc: sc.cube_stack(), 20),
}


@pytest.mark.parametrize("name", list(SCENES))
def test_tangents_match_tangent_oracle(abi, scenes, backend_mod, name):
    make, steps = SCENES[name]
    s = make(scenes)
    ref, got, _ = run_both(abi, backend_mod, s, steps, generic_seeds(abi, s.world()))
    check(ref, got)


def test_joint_stiffness_tangents(abi, scenes, backend_mod):
    """Finite bonds: the derivative along each bond's stiffness (the cap its
    penalty ramps to) and along every bond's stiffness at once."""
    s = scenes.brick_wall_c5(bond_stiffness=2e3, cols=4, rows=3)
    w = s.world()
    seeds = [(abi.SEED_JOINT_STIFFNESS, 0, 0, 0), (abi.SEED_JOINT_STIFFNESS, 3, 0, 1)]
    seeds += [(abi.SEED_JOINT_STIFFNESS, j, 0, 2) for j in range(w.n_joints)]
    seeds += [(abi.SEED_VELOCITY, w.n_bodies - 1, 1, 3), (abi.SEED_PENALTY_MAX, 0, 0, 4)]
    ref, got, _ = run_both(abi, backend_mod, s, 20, seeds)
    check(ref, got)
    assert np.max(np.abs(ref[1][..., 2])) > 0  # the bonds' stiffness does move the wall


def test_c5_wall_gradient(abi, scenes, backend_mod):
    g = json.load(open(GOLDEN))
    th = np.array(g["theta"])
    s = scenes.brick_wall_c5(mu=float(th[3]), sphere_velocity=tuple(float(v) for v in th[:3]))
    w = s.world()
    params = c5.params_of(abi, s, th, abi.ORDER_PRIORITY)
    ref, got, gpu = run_both(abi, backend_mod, s, c5.STEPS, c5.seeds(abi, s, w), params)
    check(ref, got, pos_tol=2e-6, tan_rel=2e-5)
    gpos, gtan, _ = got
    L, grad = c5.gradient_from_tangents(s, w, gpos, gtan, th)
    assert L == pytest.approx(g["objective"], rel=1e-6)
    np.testing.assert_allclose(grad, g["tangent"], rtol=2e-4, atol=1e-9)
    # the backward: one vector-Jacobian product with dL/dpos
    vjp = gpu.adjoint_backward(c5.upstream(s, w, gpos))
    vjp[4] *= th[4]
    np.testing.assert_allclose(vjp, grad, rtol=1e-12, atol=1e-18)
    fd = g["differences"][repr(c5.H[1])]
    assert abs(grad[1] - fd[1]) <= 0.05 * abs(fd[1])
    assert grad[4] == 0.0  # no bond reaches the cap


def test_bad_seeds_are_rejected(abi, scenes, backend_mod):
    s = scenes.cube_stack(n=3)
    gpu = backend_mod.GpuBackend(abi.default_params(**s.params))
    for bad in ([(abi.SEED_VELOCITY, 99, 0, 0)], [(abi.SEED_VELOCITY, 0, 3, 0)], [(abi.SEED_FRICTION, 0, 0, 5)],
                [(abi.SEED_JOINT_STIFFNESS, 0, 0, 0)], [(7, 0, 0, 0)]):
        with pytest.raises(backend_mod.AvbdError) as e:
            gpu.adjoint_forward(s.world(), 1, bad)
        assert e.value.code == abi.AVBD_ERR_ARG


def test_autograd_function_gives_the_wall_gradient(abi, scenes, backend_mod):
    """The torch.autograd.Function over the C ABI: theta = the sphere's
    velocity and the bricks' friction, the loss computed in torch from the
    returned positions, loss.backward() through avbd_adjoint_backward."""
    torch = pytest.importorskip("torch")
    ag = importlib.import_module("avbd-sandbox_gb300.autograd")
    g = json.load(open(GOLDEN))
    th0 = np.array(g["theta"])
    holder = {}

    def build(th):
        s = scenes.brick_wall_c5(mu=float(th[3]), sphere_velocity=tuple(float(v) for v in th[:3]))
        w = s.world()
        holder["s"], holder["w"] = s, w
        return w, [sd for sd in c5.seeds(abi, s, w) if sd[3] < 4]

    gpu = backend_mod.GpuBackend(c5.params_of(abi, scenes.brick_wall_c5(), th0, abi.ORDER_PRIORITY))
    theta = torch.tensor(th0[:4], dtype=torch.float64, requires_grad=True)
    pos = ag.StepFunction.apply(theta, gpu, build, c5.STEPS)
    s, w = holder["s"], holder["w"]
    b0, b1 = s.meta["bricks"]
    p0 = torch.from_numpy(w.pos[b0:b1])
    loss = (pos[b0:b1] - p0).norm(dim=1).mean()
    loss.backward()
    assert float(loss.detach()) == pytest.approx(g["objective"], rel=1e-6)
    np.testing.assert_allclose(theta.grad.numpy(), g["tangent"][:4], rtol=2e-4, atol=1e-9)
    # a second forward on the same backend makes the first one's backward stale
    pos2 = ag.StepFunction.apply(theta, gpu, build, 2)
    pos3 = ag.StepFunction.apply(theta, gpu, build, 3)
    with pytest.raises(RuntimeError):
        pos2.sum().backward()
    pos3.sum().backward()
