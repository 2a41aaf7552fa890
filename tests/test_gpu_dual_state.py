"""The constraint state after a step, element by element, against the f64
oracle; breakage; and the headline configurations at their full size.

From identical inputs (the same state, rounded to what the device stores,
warm-start manifolds included) one step on each side, then every contact's
multiplier, penalty, stick flag, anchors and C0, every joint's multipliers,
penalties and broken flag, and every spring's penalty, peak strain and
broken flag are compared (tests/dual_state.py defines the errors). The
tolerances, per quantity, relative with the floors of dual_state.FLOORS:

  quantity                       max        99.9th percentile
  contact lambda, normal         3e-2       1e-3
  contact lambda, friction rows  (*)        5e-3
  contact penalty, normal        3e-2       1e-3
  contact penalty, friction      (*)        5e-3
  contact anchors rA, rB         5e-2       1e-3   (floor 1 mm)
  contact C0                     2e-5 m     -      (absolute)
  joint lambda (lin, ang)        1e-3       -
  joint penalty (lin, ang)       3e-2       -
  spring penalty                 1e-6       -
  spring peak strain             1e-3       -      (floor 1e-3)
  stick flag (loaded contacts)   1e-4 of the contacts differ
  broken joints / springs        identical sets

(*) The friction rows hold two discrete decisions, inside or outside the
Coulomb cone (the penalty ramps only inside: manifold.js:466-479) and the
clamp onto it; a contact at the cone's edge can take the other branch in
f32. At most 1e-4 of the contacts may exceed 1e-2 there.

The f32 solver's own bound on the body state: positions 1e-5 m, quaternion
components 1e-5 (2e-5 in the crushed 51,041-body pile), velocities 1e-3 m/s,
angular velocities 3e-3 rad/s.
"""
import importlib

import numpy as np
import pytest

import dual_state as ds
from oracle import Oracle

pytestmark = pytest.mark.gpu

CONTACT_MAX = {"lambda_normal": 3e-2, "penalty_normal": 3e-2, "r_a": 5e-2, "r_b": 5e-2, "c0": 2e-5}
CONTACT_P999 = {"lambda_normal": 1e-3, "lambda_tangent": 5e-3, "penalty_normal": 1e-3, "penalty_tangent": 5e-3,
                "r_a": 1e-3, "r_b": 1e-3}
FRICTION_OUTLIER = (1e-2, 1e-4)  # (relative error, largest fraction of contacts above it)
JOINT_MAX = {"lambda_lin": 1e-3, "lambda_ang": 1e-3, "penalty_lin": 3e-2, "penalty_ang": 3e-2}
SPRING_MAX = {"penalty": 1e-6, "peak_strain": 1e-3}
STICK_FRACTION = 1e-4
BODY_TOL = {"pos": 1e-5, "quat": 1e-5, "vel": 1e-3, "omega": 3e-3}


@pytest.fixture(scope="module")
def backend_mod():
    return importlib.import_module("avbd-sandbox_gb300.backend")


def params_for(abi, s, **kw):
    return abi.default_params(**s.params, body_order=abi.ORDER_PRIORITY, **kw)


def friction_outliers(got, want):
    (rg, sg), (rw, sw), _ = ds.matched_contacts(got, want)
    if len(rg) == 0:
        return 0.0
    lam = ds.rel_err(got.m_lambda[rg, sg][:, 1:], want.m_lambda[rw, sw][:, 1:], ds.FLOORS["lambda"]).max(axis=1)
    pen = ds.rel_err(got.m_penalty[rg, sg][:, 1:], want.m_penalty[rw, sw][:, 1:], ds.FLOORS["penalty"]).max(axis=1)
    return float(np.count_nonzero(np.maximum(lam, pen) > FRICTION_OUTLIER[0])) / len(rg)


def check_dual(got, want, body_tol=BODY_TOL):
    """Every per-quantity bound of the module docstring; returns the errors."""
    e = ds.all_errors(got, want)
    for k, tol in body_tol.items():
        assert e["bodies"][k] <= tol, (k, e["bodies"][k])
    c = e["contacts"]
    assert c["unmatched"] == 0
    for k, tol in CONTACT_MAX.items():
        assert c[k]["max"] <= tol, (k, c[k])
    for k, tol in CONTACT_P999.items():
        assert c[k]["p999"] <= tol, (k, c[k])
    assert friction_outliers(got, want) <= FRICTION_OUTLIER[1]
    assert c["stick_mismatch"] <= STICK_FRACTION * max(c["active"], 1), c
    j = e["joints"]
    for k, tol in JOINT_MAX.items():
        assert j[k]["max"] <= tol, (k, j[k])
    assert j["broken_mismatch"] == 0
    sp = e["springs"]
    for k, tol in SPRING_MAX.items():
        assert sp[k]["max"] <= tol, (k, sp[k])
    assert sp["broken_mismatch"] == 0
    return e


def step_both(abi, backend_mod, params, state):
    ref = Oracle(params, state)
    gpu = backend_mod.GpuBackend(params)
    gpu.pack(state)
    ref.step(1)
    gpu.step(1)
    gpu.idle()
    return ref, gpu


def check_discrete(ref, gpu, want, got):
    oa, ob = ref.pairs()
    ga, gb = gpu.read_pairs()
    assert np.array_equal(oa, ga) and np.array_equal(ob, gb), "candidate pairs differ"
    assert got.manifold_dict() == want.manifold_dict(), "manifold topology differs"
    oc, on = ref.coloring()
    gc, gn = gpu.read_coloring()
    assert gn == on and np.array_equal(gc, oc), "colouring differs"


def small_scenes(scenes):
    out = {s.name: s for s in scenes.parity_scenes()}
    out["pyramid_small"] = scenes.pyramid(layers=6)
    out["heavy_chain_small"] = scenes.heavy_chain(links=8, springs=10)
    out["spheres"] = scenes.spheres_scene()
    out["cube_stack"] = scenes.cube_stack()
    return out


@pytest.mark.parametrize("name", ["pyramid_small", "heavy_chain_small", "spheres", "cube_stack", "pyramid", "rope",
                                  "heavy_rope", "rope_angular", "static_friction", "spring", "spring_ratio"])
@pytest.mark.parametrize("warm", [0, 25])
def test_dual_state_single_step(abi, scenes, backend_mod, name, warm):
    s = small_scenes(scenes)[name]
    params = params_for(abi, s)
    o = Oracle(params, s.world())
    o.step(warm)
    ref, gpu = step_both(abi, backend_mod, params, o.state().round_to_device())
    want, got = ref.state(), gpu.read_state(manifolds=True)
    check_discrete(ref, gpu, want, got)
    check_dual(got, want)


@pytest.mark.parametrize("warm", list(range(12)))
def test_breakage_single_step(abi, scenes, backend_mod, warm):
    """Bonds breaking from step 4 on and springs tearing at steps 5 and 9
    (scene.breakage): from the oracle's state after `warm` steps, one step on
    each side breaks the same joints and tears the same springs
    (joint.js:307-316, spring.js:461-470), with the dual state in bounds."""
    s = scenes.breakage()
    params = params_for(abi, s)
    o = Oracle(params, s.world())
    o.step(warm)
    ref, gpu = step_both(abi, backend_mod, params, o.state().round_to_device())
    want, got = ref.state(), gpu.read_state(manifolds=True)
    check_discrete(ref, gpu, want, got)
    check_dual(got, want)


def test_breakage_trajectory(abi, scenes, backend_mod):
    """Both sides step the breakage scene 15 times from the same start: after
    every step the sets of broken joints and torn springs are identical, and
    by the end 8 bonds have broken and 2 springs have torn."""
    s = scenes.breakage()
    params = params_for(abi, s)
    w = s.world().round_to_device()
    ref = Oracle(params, w)
    gpu = backend_mod.GpuBackend(params)
    gpu.pack(w)
    for _ in range(15):
        ref.step(1)
        gpu.step(1)
        gpu.idle()
        want, got = ref.state(), gpu.read_state()
        assert np.array_equal(np.nonzero(want.j_broken)[0], np.nonzero(got.j_broken)[0])
        assert np.array_equal(np.nonzero(want.s_broken)[0], np.nonzero(got.s_broken)[0])
    assert int(want.j_broken.sum()) == 8 and int(want.s_broken.sum()) == 2
    st = gpu.last_stats
    assert st["joints_broken"] == 8 and st["springs_broken"] == 2


@pytest.mark.parametrize("warm", [0, 30, 100])
def test_heavy_chain_full_single_step(abi, scenes, backend_mod, warm):
    """The full joint and mass-ratio configuration: 50 hard links of 1 kg
    ending in a 26,000 kg box (FP64 factorisation path) and the 100-spring
    chain alternating 1e3 / 1e6 N/m, 20 iterations."""
    s = scenes.heavy_chain()
    params = params_for(abi, s)
    o = Oracle(params, s.world())
    o.step(warm)
    ref, gpu = step_both(abi, backend_mod, params, o.state().round_to_device())
    assert gpu.last_stats["fp64_bodies"] >= 50
    want, got = ref.state(), gpu.read_state(manifolds=True)
    check_discrete(ref, gpu, want, got)
    check_dual(got, want)


def test_heavy_chain_full_drift(abi, scenes, backend_mod):
    """The full chain configuration for 60 steps from one start: the worst
    body stays within 5e-3 m of the oracle (the chain is chaotic later on:
    over its 1000 configured steps a 1e-7 m nudge of the oracle itself grows
    to metres)."""
    s = scenes.heavy_chain()
    params = params_for(abi, s)
    w = s.world().round_to_device()
    ref = Oracle(params, w)
    gpu = backend_mod.GpuBackend(params)
    gpu.pack(w)
    ref.step(60)
    gpu.step(60)
    gpu.idle()
    want, got = ref.state(), gpu.read_state()
    dyn = want.mass > 0
    assert np.max(np.abs(got.pos[dyn] - want.pos[dyn])) < 5e-3


def test_pile_batch_slice(abi, scenes, backend_mod):
    """16 scenes of the batched workload (64..8,192 random boxes each, 25,272
    bodies) in one context, advanced 120 steps on the device into their
    settled piles; one more step of the whole batch from that state equals
    each scene's own oracle step: manifolds, colouring, body and dual state."""
    parts = scenes.pile_batch()[:16]
    batch = scenes.batch_worlds([p.world() for p in parts])
    params = abi.default_params(gravity=-9.81, iterations=10, body_order=abi.ORDER_PRIORITY)
    gpu = backend_mod.GpuBackend(params)
    gpu.pack(batch)
    gpu.step(120)
    gpu.idle()
    state = gpu.read_state(manifolds=True).round_to_device()
    gpu.destroy()
    gpu = backend_mod.GpuBackend(params)
    gpu.pack(state)
    gpu.step(1)
    gpu.idle()
    got_all = gpu.read_state(manifolds=True)
    gc, _ = gpu.read_coloring()
    contacts = 0
    for k in range(len(parts)):
        ref = Oracle(params, ds.scene_slice(state, k))
        ref.step(1)
        want, got = ref.state(), ds.scene_slice(got_all, k)
        assert got.manifold_dict() == want.manifold_dict(), k
        oc, _ = ref.coloring()
        b0, b1 = int(state.scene_start[k]), int(state.scene_start[k + 1])
        assert np.array_equal(gc[b0:b1], oc), k
        contacts += check_dual(got, want)["contacts"]["count"]
    assert contacts > 40000


def test_crushed_pyramid_single_step(abi, scenes, backend_mod):
    """The dense pile at its size: the 53-layer pyramid (51,039 cubes, the
    sphere, the ground) advanced 150 steps on the device into the crushed
    pile (about 3M contacts, 47 colours), then one step on each side from
    that state: the same 2.9M candidate pairs, manifolds, feature IDs and
    colouring, and the body and dual state within the bounds above."""
    s = scenes.pyramid()
    params = params_for(abi, s)
    gpu = backend_mod.GpuBackend(params)
    gpu.pack(s.world())
    gpu.step(150)
    gpu.idle()
    state = gpu.read_state(manifolds=True).round_to_device()
    gpu.destroy()
    assert state.m_count > 500000
    ref, gpu = step_both(abi, backend_mod, params, state)
    want, got = ref.state(), gpu.read_state(manifolds=True)
    check_discrete(ref, gpu, want, got)
    e = check_dual(got, want, dict(BODY_TOL, quat=2e-5))
    assert e["contacts"]["count"] > 2000000
