"""The f64 oracle against contracts of the reference's headless GPU tests that
describe the CPU engine's behaviour too:

  test/gpu_headless.mjs:252-286  two spheres whose grid query spans a
      hash-colliding cell: exactly one pair, one manifold, one contact
  test/gpu_headless.mjs:753-775  a 3x3x1 box turned 45 degrees on another:
      the widest manifold after 30 steps holds the SAT maximum of 8 contacts
  test/gpu_headless.mjs:832-860  a settled stack of 6 cubes: after 150 steps
      the peak contact penalty exceeds 100 x penaltyMin (the warm start of
      Eq. 19 carries the penalty across steps)
  test/gpu_headless.mjs:1566-1635, 1713-1771  the colouring of a churning
      pile with a jointed chain and a spring, after 90 steps: statics take no
      colour, every dynamic body one colour below the cap, and no two bodies
      sharing a joint, spring or contact share a colour
  test/gpu_headless.mjs:1666-1711  a 40-link cable between two fixed anchors:
      no joint joins two bodies of one colour after 4 steps, and the state is
      finite after 60
"""
import math

import numpy as np

from oracle import Oracle


def hash_twin(scenes):
    s = scenes.Scene("hash_twin")
    s.params = dict(gravity=0.0, iterations=0, broadphase=1)
    s.sphere(1.0, 1.0, 0.5, (0.0, -0.02, -0.02))
    s.sphere(1.0, 1.0, 0.5, (0.0, 0.02, 0.02))
    return s


def octagon_stack(scenes):
    s = scenes.Scene("octagon_stack")
    s.params = dict(gravity=-10.0)
    s.box((60.0, 60.0, 2.0), 0.0, 0.5, (0.0, 0.0, -1.0))
    s.box((3.0, 3.0, 1.0), 1.0, 0.5, (0.0, 0.0, 0.5))
    s.box((3.0, 3.0, 1.0), 1.0, 0.5, (0.0, 0.0, 1.5), quat=scenes.axis_angle((0.0, 0.0, 1.0), math.pi / 4))
    return s


def cube_column(scenes):
    s = scenes.Scene("cube_column")
    s.params = dict(gravity=-10.0)
    s.box((60.0, 60.0, 2.0), 0.0, 0.5, (0.0, 0.0, -1.0))
    for i in range(6):
        s.box((1.0, 1.0, 1.0), 1.0, 0.5, (0.0, 0.0, 0.5 + i * 1.02))
    return s


def test_hash_twin_single_pair(abi, scenes):
    s = hash_twin(scenes)
    o = Oracle(abi.default_params(**s.params), s.world())
    o.step(1)
    a, b = o.pairs()
    assert len(a) == 1
    md = o.state().manifold_dict()
    assert list(md) == [(1, 0)] and md[(1, 0)][0] == 1


def test_maximum_width_manifold(abi, scenes):
    s = octagon_stack(scenes)
    o = Oracle(abi.default_params(**s.params), s.world())
    o.step(30)
    widest = max(c for c, _ in o.state().manifold_dict().values())
    assert widest == 8


def test_warm_start_accumulates_penalty(abi, scenes):
    s = cube_column(scenes)
    params = abi.default_params(**s.params)
    o = Oracle(params, s.world())
    o.step(150)
    st = o.state()
    live = st.m_num_contacts[:st.m_count] > 0
    assert live.any()
    peak = max(float(np.max(st.m_penalty[m, :st.m_num_contacts[m]])) for m in np.where(live)[0])
    assert peak > 100 * params.penalty_min


def colour_scene(scenes):
    s = scenes.Scene("colour_scene")
    s.params = dict(gravity=-10.0)
    s.box((60.0, 60.0, 2.0), 0.0, 0.5, (0.0, 0.0, -1.0))
    for x in range(-2, 3):
        for y in range(-2, 3):
            for k in range(2):
                s.box((0.9, 0.9, 0.9), 1.0, 0.5, (x * 0.95, y * 0.95, 0.5 + k * 0.95))
    prev = None
    for i in range(6):
        b = s.box((0.8, 0.4, 0.4), 0.0 if i == 0 else 1.0, 0.5, (i * 1.4 - 4, 6.0, 9.0))
        if prev is not None:
            s.joint(prev, b, (0.7, 0.0, 0.0), (-0.7, 0.0, 0.0), math.inf, math.inf)
        prev = b
    a = s.box((1.0, 1.0, 1.0), 1.0, 0.5, (4.0, 6.0, 9.0))
    c = s.box((1.0, 1.0, 1.0), 1.0, 0.5, (6.0, 6.0, 9.0))
    s.spring(a, c, (0.5, 0.0, 0.0), (-0.5, 0.0, 0.0), 800.0, 1.5)
    return s


def cable(scenes):
    s = scenes.Scene("cable")
    s.params = dict(gravity=-10.0, iterations=14)
    anchor_a = s.box((0.5, 0.5, 0.5), 0.0, 0.5, (0.0, 0.0, 20.0))
    prev, prev_anchor = anchor_a, (0.0, 0.0, 0.0)
    for k in range(40):
        bar = s.box((0.98, 0.16, 0.16), 3.0, 0.5, (k + 0.5, 0.0, 20.0))
        s.joint(prev, bar, prev_anchor, (-0.5, 0.0, 0.0))
        prev, prev_anchor = bar, (0.5, 0.0, 0.0)
    anchor_b = s.box((0.5, 0.5, 0.5), 0.0, 0.5, (40.0, 0.0, 20.0))
    s.joint(anchor_b, prev, (0.0, 0.0, 0.0), prev_anchor)
    return s


def constraint_edges(s, state):
    edges = [(j[0], j[1]) for j in s.joints] + [(sp[0], sp[1]) for sp in s.springs]
    edges += list(state.manifold_dict())
    return edges


def test_colouring_contracts(abi, scenes):
    s = colour_scene(scenes)
    params = abi.default_params(**s.params, body_order=abi.ORDER_PRIORITY)
    o = Oracle(params, s.world())
    o.step(90)
    colour, n = o.coloring()
    st = o.state()
    dyn = st.mass > 0
    assert np.all(colour[~dyn] == -1)
    assert np.all((colour[dyn] >= 0) & (colour[dyn] < n)) and n <= 64
    bad = [(a, b) for a, b in constraint_edges(s, st)
           if a >= 0 and b >= 0 and dyn[a] and dyn[b] and colour[a] == colour[b]]
    assert not bad


def test_cable_colouring_conflict_free(abi, scenes):
    s = cable(scenes)
    params = abi.default_params(**s.params, body_order=abi.ORDER_PRIORITY)
    o = Oracle(params, s.world())
    o.step(4)
    colour, _ = o.coloring()
    dyn = o.state().mass > 0
    same = [(a, b) for a, b, *_ in s.joints if dyn[a] and dyn[b] and colour[a] == colour[b]]
    assert not same
    o.step(56)
    assert np.all(np.isfinite(o.state().pos))

