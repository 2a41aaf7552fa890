"""The element-wise comparison of tests/dual_state.py, on the CPU: a world
against itself has no error, and a mistake planted in an oracle state (one
contact multiplier, one joint's broken flag, one spring's peak strain) is
reported where it was planted."""
import numpy as np

import dual_state as ds
from oracle import Oracle


def test_identical_and_planted(abi, scenes):
    s = scenes.breakage()
    params = abi.default_params(**s.params, body_order=abi.ORDER_PRIORITY)
    o = Oracle(params, s.world())
    o.step(6)
    want = o.state()
    e = ds.all_errors(want, want)
    assert e["contacts"]["lambda_normal"]["max"] == 0 and e["contacts"]["unmatched"] == 0
    assert e["joints"]["broken_mismatch"] == 0 and e["joints"]["broken"] == 4
    got = want.copy()
    got.m_lambda[3, 0, 0] *= 1.01
    got.j_broken[0] = 1 - got.j_broken[0]
    got.s_peak_strain[2] += 1e-3
    e = ds.all_errors(got, want)
    lam = abs(want.m_lambda[3, 0, 0])
    assert abs(e["contacts"]["lambda_normal"]["max"] - 0.01 * lam / max(lam, 1.0)) < 1e-12
    assert e["joints"]["broken_mismatch"] == 1
    assert abs(e["springs"]["peak_strain"]["max"] - 1e-3 / max(abs(want.s_peak_strain[2]), 1e-3)) < 1e-9


def test_scene_slice_of_one_scene(abi, scenes):
    s = scenes.random_pile(200, seed=5)
    params = abi.default_params(**s.params, body_order=abi.ORDER_PRIORITY)
    o = Oracle(params, s.world())
    o.step(90)
    w = o.state()
    part = ds.scene_slice(w, 0)
    assert part.manifold_dict() == w.manifold_dict() and np.array_equal(part.pos, w.pos)
