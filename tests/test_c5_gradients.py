"""The differentiable wall's reference gradient on the f64 oracle (CPU).

Pins the objective and its central differences (tests/golden/c5_gradients.json,
written by tests/golden/make_c5_gradients.py) and checks that they are a valid
reference: between h = 1e-4 and h = 5e-5 the derivatives along the sphere's
y and z velocity agree within 2 %, along mu within 5 %; along x, the wall's
symmetry axis, the difference is noise under 10 % of the y derivative; the
penalty cap, which no bond reaches, has a derivative of exactly zero.
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
    return {"objective": c5.objective(abi, scenes, th, c5.STEPS),
            "differences": {h: c5.central_differences(abi, scenes, th, c5.STEPS, h) for h in c5.H}}


def test_matches_golden(computed):
    g = json.load(open(GOLDEN))
    assert g["steps"] == c5.STEPS
    assert computed["objective"] == pytest.approx(g["objective"], rel=1e-12)
    for h in c5.H:
        np.testing.assert_allclose(computed["differences"][h], g["differences"][repr(h)], rtol=1e-9, atol=1e-15)


def test_differences_converge(computed):
    a, b = computed["differences"][c5.H[0]], computed["differences"][c5.H[1]]
    vx, vy, vz, mu, cap = range(5)
    for i, tol in ((vy, 0.02), (vz, 0.02), (mu, 0.05)):
        assert abs(a[i] - b[i]) <= tol * abs(b[i]), (c5.NAMES[i], a[i], b[i])
    assert abs(a[vx]) < 0.1 * abs(a[vy]) and abs(b[vx]) < 0.1 * abs(b[vy])
    assert a[cap] == 0.0 and b[cap] == 0.0
