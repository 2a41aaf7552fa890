"""The differentiable wall's reference gradient on the f64 oracle (CPU).

Pins the objective, its central differences and its exact derivative from
the tangent oracle (tests/golden/c5_gradients.json, written by
tests/golden/make_c5_gradients.py), and checks that they are a valid
reference: between h = 1e-4 and h = 5e-5 the derivatives along the sphere's
y and z velocity agree within 2 %, along mu within 5 %; along x (the sphere
strikes near the wall's middle) the difference is under 10 % of the y
derivative; the penalty cap, which no bond reaches, has a derivative of
exactly zero. The tangent oracle's values are the f64 oracle's, bit for bit,
and its derivative agrees with the differences: along y within 0.1 %, along
z and mu within the differences' own spread (3 %, 6 %).
"""
import json
import os

import numpy as np
import pytest

import c5_gradients as c5

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "c5_gradients.json")


@pytest.fixture(scope="module")
def computed():
    abi, scenes = c5.modules()
    th = c5.theta0(abi)
    L_t, g_t = c5.tangent_gradient(abi, scenes, th, c5.STEPS)
    return {"objective": c5.objective(abi, scenes, th, c5.STEPS),
            "differences": {h: c5.central_differences(abi, scenes, th, c5.STEPS, h) for h in c5.H},
            "tangent_objective": L_t, "tangent": g_t}


def test_matches_golden(computed):
    g = json.load(open(GOLDEN))
    assert g["steps"] == c5.STEPS
    assert computed["objective"] == pytest.approx(g["objective"], rel=1e-12)
    for h in c5.H:
        np.testing.assert_allclose(computed["differences"][h], g["differences"][repr(h)], rtol=1e-9, atol=1e-15)
    np.testing.assert_allclose(computed["tangent"], g["tangent"], rtol=1e-9, atol=1e-15)


def test_differences_converge(computed):
    a, b = computed["differences"][c5.H[0]], computed["differences"][c5.H[1]]
    vx, vy, vz, mu, cap = range(5)
    for i, tol in ((vy, 0.02), (vz, 0.02), (mu, 0.05)):
        assert abs(a[i] - b[i]) <= tol * abs(b[i]), (c5.NAMES[i], a[i], b[i])
    assert abs(a[vx]) < 0.1 * abs(a[vy]) and abs(b[vx]) < 0.1 * abs(b[vy])
    assert a[cap] == 0.0 and b[cap] == 0.0


def test_tangent_oracle_is_exact(computed):
    assert computed["tangent_objective"] == computed["objective"]  # the same double operations
    t, fd = computed["tangent"], computed["differences"][c5.H[1]]
    vx, vy, vz, mu, cap = range(5)
    assert abs(t[vy] - fd[vy]) <= 1e-3 * abs(fd[vy])
    assert abs(t[vz] - fd[vz]) <= 0.03 * abs(fd[vz])
    assert abs(t[mu] - fd[mu]) <= 0.06 * abs(fd[mu])
    assert abs(t[vx]) < 0.1 * abs(t[vy])
    assert t[cap] == 0.0


@pytest.mark.parametrize("name", ["cube_stack", "heavy_chain", "brick_wall_c5", "spheres"])
def test_tangent_values_follow_f64(name):
    from oracle import Oracle, TangentOracle

    abi, scenes = c5.modules()
    s = {"cube_stack": scenes.cube_stack, "heavy_chain": lambda: scenes.heavy_chain(links=4, springs=4),
         "brick_wall_c5": scenes.brick_wall_c5, "spheres": scenes.spheres_scene}[name]()
    params = abi.default_params(**s.params)
    a, b = Oracle(params, s.world()), TangentOracle(params, s.world())
    a.step(20)
    b.step(20)
    sa, sb = a.state(), b.state()
    assert np.array_equal(sa.pos, sb.pos) and np.array_equal(sa.quat, sb.quat) and np.array_equal(sa.vel, sb.vel)



def test_contact_geometry_tangents_matter():
    """Why an adjoint must differentiate the narrow phase: holding the contact
    bases and anchors constant within each step (C0 still following the poses)
    moves the v0_y derivative by far more than the 5 % tolerance."""
    from oracle import TangentOracle

    abi, scenes = c5.modules()
    th = c5.theta0(abi)
    exact = c5.tangent_gradient(abi, scenes, th, c5.STEPS)[1]
    try:
        TangentOracle.freeze_geometry(3)
        frozen = c5.tangent_gradient(abi, scenes, th, c5.STEPS)[1]
    finally:
        TangentOracle.freeze_geometry(0)
    assert abs(frozen[1] - exact[1]) > 0.2 * abs(exact[1])
