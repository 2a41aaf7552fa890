"""CUDA backend vs the f64 oracle, through the C ABI.

From identical inputs (the oracle's state rounded to what the device stores)
one step on each side must give:
  * the same candidate pair set                      (bit-exact)
  * the same manifolds: pairs, contact counts and feature IDs (bit-exact)
  * the same colouring as the oracle's integer-priority greedy colouring,
    which is also the order the oracle replays (AVBD_ORDER_PRIORITY)
  * body states within the FP32 tolerance below
Tolerances: positions 1e-5 m (the FP32 single-step position bound), orientation
components 1e-5, velocities 1e-3 m/s (= 1e-5 m / dt + rounding of delta/dt).
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


def scene_list(scenes):
    out = {s.name: s for s in scenes.parity_scenes()}
    out["cube_stack"] = scenes.cube_stack()
    out["spheres"] = scenes.spheres_scene()
    out["pyramid_small"] = scenes.pyramid(layers=6)
    out["heavy_chain_small"] = scenes.heavy_chain(links=8, springs=10)
    out["brick_wall_small"] = scenes.brick_wall(cols=6, rows=4)
    return out


SCENES = ["ground", "spinner", "stack", "stack_ratio", "pyramid", "rope", "heavy_rope", "rope_angular",
          "static_friction", "spring", "spring_ratio", "tumble", "cube_stack", "spheres", "pyramid_small",
          "heavy_chain_small", "brick_wall_small"]


def params_for(abi, s, **kw):
    return abi.default_params(**s.params, body_order=abi.ORDER_PRIORITY, **kw)


def compare_step(abi, backend_mod, s, warm_steps, **kw):
    params = params_for(abi, s, **kw)
    o = Oracle(params, s.world())
    o.step(warm_steps)
    state = o.state().round_to_device()
    ref = Oracle(params, state)
    gpu = backend_mod.GpuBackend(params)
    gpu.pack(state)
    ref.step(1)
    gpu.step(1)
    gpu.idle()
    return ref, gpu


@pytest.mark.parametrize("name", SCENES)
@pytest.mark.parametrize("warm", [0, 25])
@pytest.mark.parametrize("schedule", [0, 1])
def test_single_step_parity(abi, scenes, backend_mod, name, warm, schedule):
    s = scene_list(scenes)[name]
    ref, gpu = compare_step(abi, backend_mod, s, warm, schedule=schedule)

    oa, ob = ref.pairs()
    ga, gb = gpu.read_pairs()
    assert np.array_equal(oa, ga) and np.array_equal(ob, gb), "candidate pairs differ"

    want = ref.state()
    got = gpu.read_state(manifolds=True)
    assert got.manifold_dict() == want.manifold_dict(), "manifold topology differs"

    oc, on = ref.coloring()
    gc, gn = gpu.read_coloring()
    assert gn == on and np.array_equal(gc, oc), "colouring differs"

    dyn = want.mass > 0
    if dyn.any():
        assert np.max(np.abs(got.pos[dyn] - want.pos[dyn])) <= POS_TOL
        assert np.max(np.abs(got.quat[dyn] - want.quat[dyn])) <= QUAT_TOL
        assert np.max(np.abs(got.vel[dyn] - want.vel[dyn])) <= VEL_TOL
    assert np.all(np.isfinite(got.pos))


@pytest.mark.parametrize("name", SCENES)
def test_reference_step_schedule(abi, scenes, backend_mod, name):
    """The reference's own GPU-vs-CPU harness (src/app/gputest.js:91-96,
    139-166): from one start, after step s the worst body error, relative with
    a floor of 1 (positions) and absolute (quaternion components), stays within
    [3e-4, 1e-3, 4e-3, 2e-2][s]. The oracle replays the device colouring."""
    s = scene_list(scenes)[name]
    params = params_for(abi, s)
    w = s.world().round_to_device()
    ref = Oracle(params, w)
    gpu = backend_mod.GpuBackend(params)
    gpu.pack(w)
    for step, tol in enumerate([3e-4, 1e-3, 4e-3, 2e-2]):
        ref.step(1)
        gpu.step(1)
        gpu.idle()
        want, got = ref.state(), gpu.read_state()
        dyn = want.mass > 0
        if not dyn.any():
            continue
        pos = np.abs(got.pos[dyn] - want.pos[dyn]) / np.maximum(1.0, np.abs(want.pos[dyn]))
        quat = np.abs(got.quat[dyn] - want.quat[dyn])
        worst = max(float(pos.max()), float(quat.max()))
        assert worst <= tol, f"step {step + 1}: {worst:.3e} > {tol}"


@pytest.mark.parametrize("name", ["stack", "cube_stack", "rope", "heavy_rope", "spring_ratio", "spring"])
def test_short_horizon_drift(abi, scenes, backend_mod, name):
    """Non-chaotic scenes: 30 steps from the same start stay within 5e-3 m."""
    s = scene_list(scenes)[name]
    params = params_for(abi, s)
    w = s.world().round_to_device()
    ref = Oracle(params, w)
    gpu = backend_mod.GpuBackend(params)
    gpu.pack(w)
    ref.step(30)
    gpu.step(30)
    gpu.idle()
    want, got = ref.state(), gpu.read_state()
    dyn = want.mass > 0
    assert np.max(np.abs(got.pos[dyn] - want.pos[dyn])) < 5e-3


def test_batched_scenes_match_individual_oracles(abi, scenes, backend_mod):
    """A batch of unrelated scenes in one world steps exactly like each scene
    alone: same colouring as each scene's own oracle, body states within the
    reference harness's per-step schedule (src/app/gputest.js:91-96)."""
    parts = [scenes.cube_stack(n=6, seed=3), scenes.parity_scenes()[2], scenes.spheres_scene(),
             scenes.random_pile(40, seed=7)]
    params = abi.default_params(gravity=-9.81, iterations=10, body_order=abi.ORDER_PRIORITY)
    worlds = [p.world().round_to_device() for p in parts]
    batch = scenes.batch_worlds(worlds)
    gpu = backend_mod.GpuBackend(params)
    gpu.pack(batch)
    refs = [Oracle(params, w) for w in worlds]
    for step, tol in enumerate([3e-4, 1e-3, 4e-3]):
        gpu.step(1)
        gpu.idle()
        got = gpu.read_state()
        gc, _ = gpu.read_coloring()
        start = 0
        for w, ref in zip(worlds, refs):
            ref.step(1)
            want = ref.state()
            n = w.n_bodies
            dyn = want.mass > 0
            err = np.abs(got.pos[start:start + n][dyn] - want.pos[dyn]) / np.maximum(1.0, np.abs(want.pos[dyn]))
            assert err.max() <= tol, (step, float(err.max()))
            oc, _ = ref.coloring()
            assert np.array_equal(gc[start:start + n], oc)
            start += n


@pytest.mark.parametrize("schedule", [0, 1])
def test_determinism(abi, scenes, backend_mod, schedule):
    s = scenes.pyramid(layers=8)
    params = params_for(abi, s, schedule=schedule)
    outs = []
    for _ in range(2):
        gpu = backend_mod.GpuBackend(params)
        gpu.pack(s.world())
        gpu.step(20)
        gpu.idle()
        outs.append(gpu.read_state().pos.copy())
    assert np.array_equal(outs[0], outs[1])


def test_arena_regrow_preserves_results(abi, scenes, backend_mod):
    """Overflow-driven regrow (src/physics/gpu/backend.js:1683-1739): with a
    candidate arena sized just above the first step's need, the library grows
    it ahead of overflow; with one far below it (1 candidate per body), the
    first step overflows, is skipped on the device, and runs again after the
    regrow. Either way the warm-start manifolds carry over and the trajectory
    is bit-identical to a run with ample capacity."""
    s = scenes.pyramid(layers=10)
    outs = []
    for cap in (0, 9, 1):
        params = abi.default_params(**s.params, body_order=abi.ORDER_PRIORITY, max_pairs_per_body=cap)
        gpu = backend_mod.GpuBackend(params)
        gpu.pack(s.world())
        gpu.step(40)
        gpu.idle()
        assert gpu.last_stats["overflow"] == 0
        outs.append(gpu.read_state().pos.copy())
    assert np.array_equal(outs[0], outs[1])
    assert np.array_equal(outs[0], outs[2])


def test_overflow_retry_from_a_packed_pile(abi, scenes, backend_mod):
    """A state packed with more warm-start manifolds than the default arena's
    candidate headroom (a settled 12-layer pyramid, capacity 2 candidates per
    body): the first step overflows mid-step, is skipped and redone after the
    regrow, and equals the oracle's step from the same state."""
    s = scenes.pyramid(layers=12)
    params = params_for(abi, s)
    o = Oracle(params, s.world())
    o.step(60)
    state = o.state().round_to_device()
    ref = Oracle(params, state)
    ref.step(1)
    gpu = backend_mod.GpuBackend(params_for(abi, s, max_pairs_per_body=2))
    gpu.pack(state)
    gpu.step(1)
    gpu.idle()
    assert gpu.last_stats["overflow"] == 0 and gpu.last_stats["steps"] == 1
    want, got = ref.state(), gpu.read_state(manifolds=True)
    assert got.manifold_dict() == want.manifold_dict()
    dyn = want.mass > 0
    assert np.max(np.abs(got.pos[dyn] - want.pos[dyn])) <= POS_TOL


def test_schedules_agree(abi, scenes, backend_mod):
    """The colour-phase and wavefront schedules run the same per-body
    updates in the same dependency order: bit-identical trajectories at the
    same lanes per body (the group width sets the order of the sums)."""
    s = scenes.pyramid(layers=12)
    outs = []
    for schedule in (0, 1):
        gpu = backend_mod.GpuBackend(params_for(abi, s, schedule=schedule, lanes_per_body=32))
        gpu.pack(s.world())
        gpu.step(30)
        gpu.idle()
        outs.append(gpu.read_state())
    assert np.array_equal(outs[0].pos, outs[1].pos)
    assert np.array_equal(outs[0].quat, outs[1].quat)


def box_pairs_scene(scenes, n_pairs=2400, seed=3):
    """Isolated box pairs near contact, in five families that stress the SAT
    and clipping decisions: random poses; exactly aligned stacks (tied face
    axes, vertices on the clip planes); a 45-degree yaw (tied incident faces);
    near-parallel edges around the 1e-3 rad axis-length threshold; crossed
    45-degree edges (edge-edge contacts)."""
    rng = np.random.default_rng(seed)
    s = scenes.Scene("box_pairs")
    s.params = dict(gravity=0.0, iterations=4)
    side = int(np.ceil(np.sqrt(n_pairs)))
    ident = (0.0, 0.0, 0.0, 1.0)
    for i in range(n_pairs):
        base = np.array([(i % side) * 9.0, (i // side) * 9.0, 5.0])
        ha = rng.uniform(0.2, 1.0, 3)
        hb = rng.uniform(0.2, 1.0, 3)
        fam = i % 5
        qa, qb = ident, ident
        off = np.zeros(3)
        if fam == 0:
            qa = scenes.axis_angle(rng.normal(size=3), rng.uniform(0, np.pi))
            qb = scenes.axis_angle(rng.normal(size=3), rng.uniform(0, np.pi))
            d = rng.normal(size=3)
            off = d / np.linalg.norm(d) * rng.uniform(0.3, 1.0) * (np.linalg.norm(ha) + np.linalg.norm(hb))
        else:
            pen = [0.0, 1e-3, 0.02, -1e-3][rng.integers(4)]
            lateral = [0.0, 0.0, 0.25][rng.integers(3)] * rng.uniform(-1, 1, 2)
            if fam == 2:
                qb = scenes.axis_angle((0.0, 0.0, 1.0), np.pi / 4)
            elif fam == 3:
                eps = [1e-4, 9.99e-4, 1e-3, 1.001e-3, 1e-2][rng.integers(5)]
                qb = scenes.axis_angle(rng.normal(size=3), eps)
            elif fam == 4:
                qa = scenes.axis_angle((1.0, 0.0, 0.0), np.pi / 4)
                qb = scenes.axis_angle((0.0, 1.0, 0.0), np.pi / 4)
                pen = pen * 0.5
            za = ha[2] if fam != 4 else (ha[1] + ha[2]) / np.sqrt(2)
            zb = hb[2] if fam != 4 else (hb[0] + hb[2]) / np.sqrt(2)
            off = np.array([lateral[0], lateral[1], za + zb - pen])
        s.box(2 * ha, 500.0, 0.5, tuple(base), quat=qa)
        s.box(2 * hb, 500.0, 0.5, tuple(base + off), quat=qb)
    return s


@pytest.mark.parametrize("seed", [3, 4])
def test_narrowphase_stress_topology(abi, scenes, backend_mod, seed):
    """Thousands of isolated box pairs: the device's manifolds (pairs, contact
    counts, feature IDs) equal the oracle's exactly, and so do the pairs."""
    s = box_pairs_scene(scenes, seed=seed)
    ref, gpu = compare_step(abi, backend_mod, s, 0)
    oa, ob = ref.pairs()
    ga, gb = gpu.read_pairs()
    assert np.array_equal(oa, ga) and np.array_equal(ob, gb)
    want = ref.state().manifold_dict()
    got = gpu.read_state(manifolds=True).manifold_dict()
    assert len(want) > 1000
    assert got == want


@pytest.mark.parametrize("schedule", [0, 1])
def test_more_colors_than_a_word(abi, scenes, backend_mod, schedule):
    """A complete constraint graph of 72 bodies needs 72 colours, past the
    64 of one bit word: the device colouring equals the oracle's greedy
    priority colouring, one step matches the oracle, and 30 more steps run
    without error within the reference harness's tolerance at step 4
    (src/app/gputest.js:91-96) and the 30-step drift bound."""
    s = scenes.joint_clique()
    ref, gpu = compare_step(abi, backend_mod, s, 0, schedule=schedule)
    oc, on = ref.coloring()
    gc, gn = gpu.read_coloring()
    assert on == 72 and gn == on and np.array_equal(gc, oc)
    want, got = ref.state(), gpu.read_state()
    dyn = want.mass > 0
    assert np.max(np.abs(got.pos[dyn] - want.pos[dyn])) <= POS_TOL
    assert np.max(np.abs(got.quat[dyn] - want.quat[dyn])) <= QUAT_TOL
    ref.step(29)
    gpu.step(29)
    gpu.idle()
    want, got = ref.state(), gpu.read_state()
    assert gpu.last_stats["colors"] == 72 and gpu.last_stats["overflow"] == 0
    assert np.max(np.abs(got.pos[dyn] - want.pos[dyn])) < 5e-3
