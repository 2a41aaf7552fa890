"""Pin the f64 oracle against the reference's closed-form tests.

Each test restates one known answer from the reference's own test suite,
with its tolerance:
  test/analytic.mjs:43-56    free fall = exact BDF1 trajectory, rel < 1e-12
  test/analytic.mjs:62-71    ballistic flight keeps horizontal momentum, < 1e-12
  test/analytic.mjs:76-90    cuboid inertia tensor, rel < 1e-15
  test/analytic.mjs:102-135  static friction threshold = atan(sqrt(mu_a mu_b)) +- 1.5 deg
  test/analytic.mjs:146-170  impact momentum residual ratio (10 vs 40 iterations) > 100
  test/analytic.mjs:185-209  resting sink = collision margin +- 2e-4; < 1e-3 with no margin
  test/analytic.mjs:228-274  torque-free L drift > 1% (characterisation); cube forms agree < 1e-12
  test/analytic.mjs:298-396  rotated inertia conserves L > 10x better; isotropic forms agree < 1e-15
  test/fixtures.mjs:62-135   spring_ladder built at its analytic equilibrium does not drift
  test/fixtures.mjs:170-256  plate_pendulum period vs the compound-pendulum closed form
  test/spheres.mjs           sphere mass/inertia, sphere-OBB distances, features, settling
"""
import math

import numpy as np
import pytest

from oracle import Oracle


def run(scene, params, steps):
    o = Oracle(params, scene.world())
    o.step(steps)
    return o


def test_free_fall_bdf1(scenes, abi):
    s = scenes.Scene()
    s.box((1, 1, 1), 1, 0.5, (0, 0, 100))
    p = abi.default_params()
    N = 120
    st = run(s, p, N).state()
    z_exact = 100 + p.gravity * p.dt * p.dt * ((N * (N + 1)) / 2)
    v_exact = N * p.gravity * p.dt
    assert abs(st.pos[0, 2] - z_exact) / abs(z_exact) < 1e-12
    assert abs(st.vel[0, 2] - v_exact) / abs(v_exact) < 1e-12


def test_ballistic_momentum(scenes, abi):
    s = scenes.Scene()
    s.box((1, 1, 1), 1, 0.5, (0, 0, 100), velocity=(3, -2, 0))
    st = run(s, abi.default_params(), 120).state()
    assert abs(st.vel[0, 0] - 3) / 3 < 1e-12
    assert abs(st.vel[0, 1] + 2) / 2 < 1e-12


def test_cuboid_inertia(scenes):
    s = scenes.Scene()
    size, density = (2, 3, 5), 7
    s.box(size, density, 0.5, (0, 0, 0))
    w = s.world()
    m = size[0] * size[1] * size[2] * density
    exact = [m * (size[1] ** 2 + size[2] ** 2) / 12, m * (size[0] ** 2 + size[2] ** 2) / 12,
             m * (size[0] ** 2 + size[1] ** 2) / 12]
    assert max(abs(w.moment[0, i] - e) / e for i, e in enumerate(exact)) < 1e-15


def test_static_friction_threshold(scenes, abi):
    mu_block, mu_ramp = 0.5, 1.0
    predicted = math.degrees(math.atan(math.sqrt(mu_block * mu_ramp)))

    def slides(deg):
        a = math.radians(deg)
        s = scenes.Scene()
        r = s.box((60, 60, 1), 0, mu_ramp, (0, 0, 6))
        s.set_orientation(r, (0, 1, 0), a)
        n = (math.sin(a), 0, math.cos(a))
        b = s.box((1, 1, 1), 1, mu_block, (n[0], 0, 6 + n[2]))
        s.set_orientation(b, (0, 1, 0), a)
        o = Oracle(abi.default_params(), s.world())
        o.step(200)
        x0, z0 = o.state().pos[1, [0, 2]]
        o.step(400)
        x1, z1 = o.state().pos[1, [0, 2]]
        return math.hypot(x1 - x0, z1 - z0) > 0.02

    lo, hi = 20.0, 50.0
    for _ in range(12):
        mid = (lo + hi) / 2
        if slides(mid):
            hi = mid
        else:
            lo = mid
    assert abs((lo + hi) / 2 - predicted) < 1.5


def test_impact_momentum_is_convergence_residual(scenes, abi):
    def momentum_error(iterations):
        s = scenes.Scene()
        s.box((1, 1, 1), 1, 0.0, (-3, 0, 0), velocity=(4, 0, 0))
        s.box((1, 1, 1), 2, 0.0, (3, 0, 0), velocity=(-1, 0, 0))
        o = Oracle(abi.default_params(gravity=0.0, iterations=iterations), s.world())
        w = s.world()
        p0 = w.mass[0] * 4 + w.mass[1] * -1
        worst = 0.0
        for _ in range(400):
            o.step(1)
            st = o.state()
            worst = max(worst, abs(w.mass[0] * st.vel[0, 0] + w.mass[1] * st.vel[1, 0] - p0))
        return worst

    assert momentum_error(10) / momentum_error(40) > 100


@pytest.mark.parametrize("thickness", [1.0, 0.2, 0.05])
def test_rest_sink_equals_margin(scenes, abi, thickness):
    s = scenes.Scene()
    s.box((400, 400, 4), 0, 0.5, (0, 0, -2))
    s.box((2, 2, thickness), 1, 0.5, (0, 0, 3))
    p = abi.default_params()
    sink = thickness / 2 - run(s, p, 900).state().pos[1, 2]
    assert abs(sink - p.collision_margin) < 2e-4


def test_rest_sink_no_margin(scenes, abi):
    s = scenes.Scene()
    s.box((400, 400, 4), 0, 0.5, (0, 0, -2))
    s.box((2, 2, 1.0), 1, 0.5, (0, 0, 3))
    sink = 0.5 - run(s, abi.default_params(collision_margin=0.0), 900).state().pos[1, 2]
    assert sink < 1e-3


def _world_L(st, w, idx):
    """Total world angular momentum about the origin with R I R^T (analytic.mjs:327-346)."""
    L = np.zeros(3)
    for i in idx:
        x, y, z, q = st.quat[i]
        R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - q * z), 2 * (x * z + q * y)],
                      [2 * (x * y + q * z), 1 - 2 * (x * x + z * z), 2 * (y * z - q * x)],
                      [2 * (x * z - q * y), 2 * (y * z + q * x), 1 - 2 * (x * x + y * y)]])
        I = R @ np.diag(w.moment[i]) @ R.T
        L += I @ st.omega[i] + w.mass[i] * np.cross(st.pos[i], st.vel[i])
    return L


def test_torque_free_rotation_characterisation(scenes, abi):
    def drift(rotated, size, steps):
        s = scenes.Scene()
        s.box(size, 1, 0.5, (0, 0, 0), omega=(1.3, 0.7, 0.4))
        w = s.world()
        o = Oracle(abi.default_params(gravity=0.0, rotated_inertia=int(rotated)), w)
        L0 = _world_L(o.state(), w, [0])
        worst = 0.0
        for _ in range(steps):
            o.step(1)
            worst = max(worst, np.linalg.norm(_world_L(o.state(), w, [0]) - L0) / np.linalg.norm(L0))
        return worst

    assert drift(True, (1, 2, 4), 600) > 0.01
    assert abs(drift(True, (1, 1, 1), 200) - drift(False, (1, 1, 1), 200)) < 1e-12


def test_rotated_inertia_conserves_impact_L(scenes, abi):
    def run_impact(rotated, iterations, size):
        s = scenes.Scene()
        a = s.box(size, 1, 0, (-2.2, 0.7, 0), velocity=(3, 0, 0))
        b = s.box(size, 1, 0, (2.2, -0.7, 0), velocity=(-3, 0, 0))
        s.b["quat"][a] = scenes.axis_angle((0.3, 0.5, 0.81), 0.9)
        s.b["quat"][b] = scenes.axis_angle((0.7, -0.2, 0.68), -1.2)
        w = s.world()
        o = Oracle(abi.default_params(gravity=0.0, iterations=iterations, rotated_inertia=int(rotated)), w)
        worst, contacted = 0.0, False
        for _ in range(120):
            before = _world_L(o.state(), w, [0, 1])
            scale = np.linalg.norm(before) or 1.0
            o.step(1)
            after = _world_L(o.state(), w, [0, 1])
            if o.stats()["contacts"] > 0:
                contacted = True
                worst = max(worst, np.linalg.norm(after - before) / scale)
        assert contacted
        return worst

    box, cube = (1, 2, 4), (1, 1, 1)
    rot10 = run_impact(True, 10, box)
    body10 = run_impact(False, 10, box)
    assert body10 / rot10 > 10
    assert run_impact(False, 240, box) / body10 > 0.5
    assert abs(run_impact(True, 10, cube) - run_impact(False, 10, cube)) < 1e-15


def test_spring_ladder_equilibrium(scenes, abi):
    """fixtures.mjs:62-135: exactly zero drift with the Eq. 16 ramp off."""
    N, REST, SIZE, TOP, g = 6, 1.0, 0.4, 12.0, 10.0
    density = 1 / (SIZE * SIZE * SIZE)
    mass = SIZE * SIZE * SIZE * density
    stiff = [1.0e6 if i % 2 == 0 else 1.0e3 for i in range(N)]
    z, analytic = TOP, []
    for i in range(N):
        z -= REST + (g * (N - i) * mass) / stiff[i]
        analytic.append(z)
    s = scenes.Scene()
    prev = s.box((0.6, 0.6, 0.6), 0, 0.5, (0, 0, TOP))
    for i in range(N):
        b = s.box((SIZE,) * 3, density, 0.5, (0, 0, analytic[i]))
        s.spring(prev, b, (0, 0, 0), (0, 0, 0), stiff[i], REST)
        prev = b
    o = Oracle(abi.default_params(), s.world())
    o.step(900)
    worst = 0.0
    for _ in range(300):
        o.step(1)
        worst = max(worst, float(np.max(np.abs(o.state().pos[1:, 2] - analytic))))
    assert worst / REST < 1e-9


def test_plate_pendulum_period(scenes, abi):
    """fixtures.mjs:170-256: compound pendulum, thin axis on the swing axis."""
    LEN, WIDE, THIN, DENSITY, OMEGA = 1.0, 1.2, 0.15, 4.0, 0.2
    PIVOT = (0, 0, 8)
    s = scenes.Scene()
    plate = s.box((LEN, WIDE, THIN), DENSITY, 0.5, (0, 0, PIVOT[2] - LEN / 2))
    s.set_orientation(plate, (1, 1, -1), 2 * math.pi / 3)
    s.joint(-1, plate, PIVOT, (-LEN / 2, 0, 0), math.inf, 0.0)
    s.b["omega"][plate] = (0.0, OMEGA, 0.0)
    w = s.world()
    o = Oracle(abi.default_params(), w)
    J = o.world_moment(plate, True)
    d, m = LEN / 2, w.mass[plate]
    period = 2 * math.pi * math.sqrt((J[1, 1] + m * d * d) / (m * 10.0 * d))
    o.step(60)
    angle = lambda st: math.atan2(st.pos[0, 0] - PIVOT[0], -(st.pos[0, 2] - PIVOT[2]))
    prev, crossings = angle(o.state()), []
    for step in range(1, 1201):
        o.step(1)
        a = angle(o.state())
        if prev < 0 <= a:
            crossings.append(step - 1 + (0 - prev) / (a - prev))
        prev = a
    assert len(crossings) >= 2
    measured = (crossings[-1] - crossings[0]) / (len(crossings) - 1) * (1 / 60)
    assert abs(measured - period) / period < 0.05


def test_sphere_mass_and_isotropic_world_inertia(scenes, abi):
    s = scenes.Scene()
    i = s.sphere(2, 3, 0.5, (0, 0, 0))
    s.b["quat"][i] = scenes.axis_angle((0.2, -0.7, 0.4), 1.37)
    w = s.world()
    assert abs(w.mass[0] - 4 * math.pi) < 1e-12
    assert np.all(np.abs(w.moment[0] - 0.4 * 4 * math.pi) < 1e-12)
    J = Oracle(abi.default_params(), w).world_moment(0, True)
    assert J[0, 0] == J[1, 1] == J[2, 2] == w.moment[0, 0]
    assert np.all(J[~np.eye(3, dtype=bool)] == 0)


@pytest.mark.parametrize("xy,expect", [(0.65, 0), (0.63, 1)])
def test_sphere_obb_curved_corner(scenes, abi, xy, expect):
    s = scenes.Scene()
    s.box((1, 1, 1), 0, 0.5, (0, 0, 0))
    s.sphere(0.4, 1, 0.5, (xy, xy, 0))
    n, *_ = Oracle(abi.default_params(), s.world()).collide(1, 0)
    assert n == expect


def test_sub_millimetre_sphere_normal(scenes, abi):
    s = scenes.Scene()
    s.sphere(0.001, 0, 0.5, (0, 0, 0))
    s.sphere(0.001, 1, 0.5, (0, 0.0008, 0))
    n, basis, _, ra, rb = Oracle(abi.default_params(), s.world()).collide(0, 1)
    assert n == 1 and abs(basis[0]) < 1e-12 and abs(basis[1] + 1) < 1e-12
    gap = basis[:3] @ ((np.array([0, 0, 0]) + ra[0]) - (np.array([0, 0.0008, 0]) + rb[0]))
    assert abs(gap - (0.0008 - 0.001)) < 1e-12


def test_sphere_obb_features_distinct(scenes, abi):
    s = scenes.Scene()
    s.box((1, 1, 1), 0, 0.5, (0, 0, 0))
    for p in [(0.55, 0, 0), (-0.55, 0, 0), (0.53, 0.53, 0), (0.53, -0.53, 0.53)]:
        s.sphere(0.2, 1, 0.5, p)
    o = Oracle(abi.default_params(), s.world())
    feats = [int(o.collide(k, 0)[2][0]) for k in range(1, 5)]
    assert len(set(feats)) == 4


def test_sphere_obb_signed_distance_sweep(scenes, abi):
    """spheres.mjs:190-241: 400 rotated boxes vs analytic signed distance."""
    state = [0x6D2B79F5]

    def random():
        state[0] = (state[0] * 1664525 + 1013904223) & 0xFFFFFFFF
        return state[0] / 0x100000000

    for sample in range(400):
        size = [0.2 + random() * 2.8 for _ in range(3)]
        center = [-2 + random() * 4 for _ in range(3)]
        axis = [random() - 0.5, random() - 0.5, random() - 0.5]
        angle = (random() - 0.5) * math.pi * 2
        radius = 0.02 + random() * 0.5
        half = [v * 0.5 for v in size]
        local = [(random() * 2 - 1) * (h + radius * 1.8) for h in half]
        clamped = [max(-h, min(h, v)) for h, v in zip(half, local)]
        outside = [v - c for v, c in zip(local, clamped)]
        od = math.sqrt(sum(x * x for x in outside))
        expected = od - radius if od > 0 else -(radius + min(h - abs(v) for h, v in zip(half, local)))
        s = scenes.Scene()
        b = s.box(size, 0, 0.5, center)
        s.set_orientation(b, axis, angle)
        q = s.b["quat"][b]
        rot = scenes._rotate(q, local)
        s.sphere(radius * 2, 1, 0.5, [c + r for c, r in zip(center, rot)])
        w = s.world()
        n, basis, _, ra, rb = Oracle(abi.default_params(), w).collide(1, 0)
        assert (n > 0) == (expected <= 0), sample
        if n:
            xa = w.pos[1] + np.array(scenes._rotate(w.quat[1], ra[0]))
            xb = w.pos[0] + np.array(scenes._rotate(w.quat[0], rb[0]))
            assert abs(basis[:3] @ (xa - xb) - expected) < 2e-10
            assert abs(np.linalg.norm(basis[:3]) - 1) < 2e-12


def test_sphere_settles_on_ground(scenes, abi):
    s = scenes.Scene()
    s.box((20, 20, 2), 0, 0.5, (0, 0, -1))
    s.sphere(1, 1, 0.5, (0, 0, 3))
    st = run(s, abi.default_params(), 180).state()
    assert abs(st.pos[1, 2] - 0.49) < 2e-4 and abs(st.vel[1, 2]) < 1e-3


def test_rolling_sphere_keeps_support_point(scenes, abi):
    s = scenes.Scene()
    s.box((100, 100, 2), 0, 1, (0, 0, -1))
    s.sphere(1, 1, 1, (0, 0, 0.49), velocity=(2, 0, 0))
    st = run(s, abi.default_params(), 180).state()
    assert abs(st.pos[1, 2] - 0.49) < 0.003 and abs(st.vel[1, 2]) < 0.01 and st.omega[1, 1] > 1
