"""The f64 oracle against the reference's settled-pile checks
(test/convergence.mjs:136-205), on the reference's own scenes restated from
src/app/scenes.js: `box_stack` (:290-310, 3 columns of 14 cubes), `pyramid`
(:244-288, two 14-layer pyramids of 1 x 0.6 x 0.6 blocks, 16 iterations) and
`card_tower` (:333-386, six levels of leaning cards and decks, friction 1.2).

Each scene settles for 300 steps, then a 120-step window measures the
penetration -C_n of every live contact (as a fraction of the smallest body
dimension) and the kinetic energy. The checks, with the reference's limits:
  * settled penetration stays small: box_stack < 2e-4, pyramid < 5e-3,
    card_tower < 1.5e-2 (maximum over the window)
  * penetration is a convergence residual: the mean at the shipped iteration
    count over the mean at 40 iterations > 5 (pyramid, card_tower)
  * the default dissipates energy: KE(last 20 steps) / KE(first 20) < 1
    (pyramid, card_tower)
  * post-stabilisation injects energy on the pyramid: that ratio > 2
"""
import math

import numpy as np
import pytest

from oracle import Oracle

SETTLE_STEPS = 300
WINDOW_STEPS = 120


def box_stack(scenes):
    s = scenes.Scene("box_stack")
    scenes.add_ground(s)
    for col in range(3):
        for i in range(14):
            s.box((1.2, 1.2, 1.2), 1.0, 0.5, ((col - 1) * 3.2, 0.0, 0.6 + i * 1.22))
    return s, {}


def pyramid(scenes):
    s = scenes.Scene("pyramid")
    scenes.add_ground(s)
    size = 14
    for y0 in (0.0, 2.2):
        for y in range(size):
            for x in range(size - y):
                s.box((1.0, 0.6, 0.6), 1.0, 0.6, (x * 1.02 + y * 0.51 - size / 2, y0, y * 0.62 + 0.31))
    return s, {"iterations": 16}


def card_tower(scenes):
    friction = 1.2
    s = scenes.Scene("card_tower")
    scenes.add_ground(s, friction)
    levels, H, T, W = 6, 2.0, 0.06, 1.4
    lean, spacing = math.radians(17.0), 2.0
    sn, cs = math.sin(lean), math.cos(lean)
    offset = (H / 2) * sn + (T / 2) * cs
    rise = (H / 2) * cs + (T / 2) * sn
    top = H * cs + T * sn
    deck_length = spacing + 0.36
    base = 0.0
    for lvl in range(levels):
        count = levels - lvl
        xs = [(i - (count - 1) / 2) * spacing for i in range(count)]
        for x in xs:
            for side in (-1, 1):
                s.box((T, W, H), 0.6, friction, (x + side * offset, 0.0, base + rise),
                      quat=scenes.axis_angle((0.0, 1.0, 0.0), -side * lean))
        base += top + 0.002
        for i in range(count - 1):
            s.box((deck_length, W, T), 0.6, friction, ((xs[i] + xs[i + 1]) / 2, 0.0, base + T / 2))
        base += T + 0.002
    return s, {}


SCENES = {"box_stack": box_stack, "pyramid": pyramid, "card_tower": card_tower}
CONFIGS = {"as shipped": {}, "iterations 40": {"iterations": 40}, "postStabilize": {"post_stabilize": 1}}


def probe(abi, scenes, scene, config):
    s, own = SCENES[scene](scenes)
    params = abi.default_params(**{**own, **config})
    w = s.world()
    o = Oracle(params, w)
    dyn = w.mass > 0
    feature = float(w.size[dyn].min())
    o.step(SETTLE_STEPS)
    pen_max, pen_mean_sum, energy = 0.0, 0.0, []
    for _ in range(WINDOW_STEPS):
        o.step(1)
        d = np.maximum(0.0, -o.contact_normal_c())
        if len(d):
            pen_max = max(pen_max, float(d.max()))
            pen_mean_sum += float(d.mean())
        st = o.state()
        v, om = st.vel[dyn], st.omega[dyn]
        e = 0.5 * np.sum(w.mass[dyn][:, None] * v * v) + 0.5 * np.sum(w.moment[dyn] * om * om)
        energy.append(e)
    ke_ratio = sum(energy[-20:]) / max(1e-30, sum(energy[:20]))
    return {"pen_max": pen_max / feature, "pen_mean": pen_mean_sum / WINDOW_STEPS / feature, "ke_ratio": ke_ratio}


@pytest.fixture(scope="module")
def measured(abi, scenes):
    want = {("box_stack", "as shipped"), ("pyramid", "as shipped"), ("card_tower", "as shipped"),
            ("pyramid", "iterations 40"), ("card_tower", "iterations 40"), ("pyramid", "postStabilize")}
    return {k: probe(abi, scenes, k[0], CONFIGS[k[1]]) for k in want}


@pytest.mark.parametrize("scene,limit", [("box_stack", 2e-4), ("pyramid", 5e-3), ("card_tower", 1.5e-2)])
def test_settled_penetration_stays_small(measured, scene, limit):
    assert measured[(scene, "as shipped")]["pen_max"] < limit


@pytest.mark.parametrize("scene", ["pyramid", "card_tower"])
def test_penetration_is_a_convergence_residual(measured, scene):
    assert measured[(scene, "as shipped")]["pen_mean"] / measured[(scene, "iterations 40")]["pen_mean"] > 5


@pytest.mark.parametrize("scene", ["pyramid", "card_tower"])
def test_default_dissipates_energy(measured, scene):
    assert measured[(scene, "as shipped")]["ke_ratio"] < 1.0


def test_post_stabilize_injects_energy(measured):
    assert measured[("pyramid", "postStabilize")]["ke_ratio"] > 2.0
