"""The f64 oracle against contracts of the reference's headless GPU tests that
describe the CPU engine's behaviour too:

  test/gpu_headless.mjs:252-286  two spheres whose grid query spans a
      hash-colliding cell: exactly one pair, one manifold, one contact
  test/gpu_headless.mjs:753-775  a 3x3x1 box turned 45 degrees on another:
      the widest manifold after 30 steps holds the SAT maximum of 8 contacts
  test/gpu_headless.mjs:832-860  a settled stack of 6 cubes: after 150 steps
      the peak contact penalty exceeds 100 x penaltyMin (the warm start of
      Eq. 19 carries the penalty across steps)
"""
import math

import numpy as np
import pytest

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
