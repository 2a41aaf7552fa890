"""Lane groups of two and four warps in the colour-phase solve, against the oracle.

A dynamic plate on the ground carries an n x n grid of cubes (2 m apart, so
each cube touches only the plate); the plate's constraint count is
4 n^2 + 4 contact sides: 148 at n = 6 (a 64-lane group), 328 at n = 9 (a
128-lane group, reduced through shared memory with named barriers). One step
from identical inputs must match the oracle as in test_gpu_parity; the
profile's mean lanes per body must follow the sizing rule (the fewest of
4..128 lanes holding four constraints each), and a fixed 32 lanes (several
staging chunks per lane for the plate) must match too.
"""
import importlib

import numpy as np
import pytest

from oracle import Oracle

pytestmark = pytest.mark.gpu

POS_TOL = 1e-5
QUAT_TOL = 1e-5
VEL_TOL = 1e-3


@pytest.fixture(scope="module")
def backend_mod():
    return importlib.import_module("avbd-sandbox_gb300.backend")


def loaded_plate(scenes, n):
    s = scenes.Scene(f"loaded_plate_{n}")
    s.params = dict(gravity=-9.81, iterations=10)
    scenes.add_ground(s, 0.6)
    side = 2.0 * n + 2.0
    s.box((side, side, 0.5), 1000.0, 0.6, (0.0, 0.0, 0.25 - 1e-3))
    for i in range(n):
        for j in range(n):
            x = (i - (n - 1) / 2) * 2.0
            y = (j - (n - 1) / 2) * 2.0
            s.box((1.0, 1.0, 1.0), 1000.0, 0.6, (x, y, 0.5 + 0.5 - 2e-3))
    return s


def expected_mean_lanes(state, lanes_fixed):
    """The sizing rule applied to each dynamic body's contact sides."""
    dyn = state.mass > 0
    sides = np.zeros(len(state.mass), np.int64)
    for (a, b), (count, _) in state.manifold_dict().items():
        for k in (a, b):
            if k >= 0 and dyn[k]:
                sides[k] += count
    if lanes_fixed:
        return lanes_fixed
    g = []
    for k in np.where(dyn)[0]:
        G = 4
        while G < 128 and 4 * G < sides[k]:
            G <<= 1
        g.append(G)
    n = len(g)
    return (sum(g) + n // 2) // n


@pytest.mark.parametrize("n", [6, 9])
@pytest.mark.parametrize("lanes", [0, 32])
def test_lane_groups_match_oracle(abi, scenes, backend_mod, n, lanes):
    s = loaded_plate(scenes, n)
    params = abi.default_params(**s.params, body_order=abi.ORDER_PRIORITY, schedule=0, lanes_per_body=lanes)
    o = Oracle(params, s.world())
    o.step(3)  # contacts and warm starts in place
    state = o.state().round_to_device()
    ref = Oracle(params, state)
    gpu = backend_mod.GpuBackend(params)
    gpu.pack(state)
    gpu.set_profiling(True)
    ref.step(1)
    gpu.step(1)
    prof = gpu.last_profile
    gpu.idle()

    want = ref.state()
    got = gpu.read_state(manifolds=True)
    assert got.manifold_dict() == want.manifold_dict(), "manifold topology differs"
    oc, on = ref.coloring()
    gc, gn = gpu.read_coloring()
    assert gn == on and np.array_equal(gc, oc), "colouring differs"
    plate_sides = sum(c for (a, b), (c, _) in want.manifold_dict().items() if 1 in (a, b))
    assert plate_sides >= 4 * n * n, "the cubes do not all rest on the plate"
    assert prof["lanes_per_body"] == expected_mean_lanes(want, lanes)

    dyn = want.mass > 0
    assert np.max(np.abs(got.pos[dyn] - want.pos[dyn])) <= POS_TOL
    assert np.max(np.abs(got.quat[dyn] - want.quat[dyn])) <= QUAT_TOL
    assert np.max(np.abs(got.vel[dyn] - want.vel[dyn])) <= VEL_TOL
