"""The remaining GpuBackend entry points, through the C ABI:
uploadColoring/overrideColoring (avbd_set_coloring), updateJointAnchor
(avbd_update_joint_anchor) and getConstraintGpuState (avbd_device_views_get)."""
import ctypes as C
import glob
import importlib

import numpy as np
import pytest

from oracle import Oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def backend_mod():
    return importlib.import_module("avbd-sandbox_gb300.backend")


def warm_state(abi, s, steps):
    params = abi.default_params(**s.params, body_order=abi.ORDER_PRIORITY)
    o = Oracle(params, s.world())
    o.step(steps)
    return params, o.state().round_to_device()


@pytest.mark.parametrize("name", ["pyramid", "stack"])
def test_uploaded_index_order_coloring(abi, scenes, backend_mod, name):
    """The reference CPU solver's colouring (greedy in index order,
    src/physics/coloring.js:43-118) of this step's graph, uploaded: the device
    uses it, and one step matches the oracle replaying the same order."""
    s = scenes.pyramid(layers=6) if name == "pyramid" else scenes.parity_scenes()[2]
    params, s0 = warm_state(abi, s, 20)
    probe = Oracle(params, s0)
    probe.step(1)
    col, ncol = probe.index_coloring()  # proper for this step's constraint graph
    dyn = s0.mass > 0
    order = [int(i) for i in sorted(np.nonzero(dyn)[0], key=lambda i: (col[i], i))]
    ref_params = abi.default_params(**s.params, body_order=abi.ORDER_EXPLICIT)
    ref = Oracle(ref_params, s0)
    ref.set_body_order(np.array(order, np.int32))
    ref.step(1)
    gpu = backend_mod.GpuBackend(params)
    gpu.pack(s0)
    gpu.set_coloring(col)
    gpu.step(1)
    gpu.idle()
    gc, gn = gpu.read_coloring()
    assert gn == ncol and np.array_equal(gc[dyn], col[dyn])
    want, got = ref.state(), gpu.read_state()
    assert np.max(np.abs(got.pos[dyn] - want.pos[dyn])) <= 1e-5
    assert np.max(np.abs(got.quat[dyn] - want.quat[dyn])) <= 1e-5


def test_improper_coloring_is_rejected(abi, scenes, backend_mod):
    s = scenes.pyramid(layers=6)
    params, s0 = warm_state(abi, s, 20)
    gpu = backend_mod.GpuBackend(params)
    gpu.pack(s0)
    gpu.set_coloring(np.zeros(s0.n_bodies, np.int32))  # neighbours share colour 0
    gpu.step(1)
    with pytest.raises(backend_mod.AvbdError) as e:
        gpu.idle()
    assert e.value.code == abi.AVBD_ERR_ARG
    # the step used the device's own colouring: it equals the oracle's priority step
    ref = Oracle(params, s0)
    ref.step(1)
    dyn = s0.mass > 0
    gc, _ = gpu.read_coloring()
    oc, _ = ref.coloring()
    assert np.array_equal(gc, oc)
    assert np.max(np.abs(gpu.read_state().pos[dyn] - ref.state().pos[dyn])) <= 1e-5
    gpu.set_coloring(None)
    gpu.step(1)
    gpu.idle()


def test_update_joint_anchor(abi, scenes, backend_mod):
    """Moving the world anchor of the chain's first joint between steps equals
    stepping a world whose joint was built at the new anchor."""
    s = scenes.heavy_chain(links=8, springs=10)
    params, s0 = warm_state(abi, s, 10)
    j = 0
    assert s0.j_body_a[j] < 0  # world-anchored
    new = s0.j_r_a[j] + np.array([0.05, -0.02, 0.03])
    moved = s0.copy()
    moved.j_r_a[j] = new
    ref = Oracle(params, moved)
    ref.step(1)
    gpu = backend_mod.GpuBackend(params)
    gpu.pack(s0)
    gpu.update_joint_anchor(j, new)
    gpu.step(1)
    gpu.idle()
    dyn = s0.mass > 0
    got, want = gpu.read_state(), ref.state()
    assert np.max(np.abs(got.pos[dyn] - want.pos[dyn])) <= 1e-5
    unmoved = Oracle(params, s0)
    unmoved.step(1)
    assert np.max(np.abs(unmoved.state().pos[dyn] - want.pos[dyn])) > 1e-4  # the move mattered
    with pytest.raises(backend_mod.AvbdError):
        gpu.update_joint_anchor(s0.n_joints, new)


def _cudart():
    for pat in ("/usr/local/cuda/lib64/libcudart.so*", "/usr/local/cuda/targets/*/lib/libcudart.so*"):
        for path in sorted(glob.glob(pat)):
            try:
                return C.CDLL(path)
            except OSError:
                continue
    return None


def test_device_views(abi, scenes, backend_mod):
    s = scenes.heavy_chain(links=8, springs=10)
    gpu = backend_mod.GpuBackend(abi.default_params(**s.params))
    w = s.world()
    gpu.pack(w)
    gpu.step(3)
    gpu.idle()
    v = gpu.device_views()
    assert v["body_count"] == w.n_bodies and v["joint_count"] == w.n_joints and v["spring_count"] == w.n_springs
    assert v["body_pos"] and v["body_quat"] and v["joint_state"] and v["spring_state"]
    rt = _cudart()
    if rt is None:
        pytest.skip("no libcudart to read device memory with")
    rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    pos = np.zeros((w.n_bodies, 4))
    assert rt.cudaMemcpy(pos.ctypes.data, v["body_pos"], pos.nbytes, 2) == 0  # device to host
    assert np.array_equal(pos[:, :3], gpu.read_state().pos)
    st = np.zeros(w.n_joints, np.int32)
    assert rt.cudaMemcpy(st.ctypes.data, v["joint_state"], st.nbytes, 2) == 0
    assert np.array_equal(st & 1, gpu.read_state().j_broken)


def test_graph_replay_is_bit_identical(abi, scenes, backend_mod):
    """Steps replayed as CUDA graphs (one per manifold-arena parity) give the
    same trajectory bit for bit as directly launched steps, through an arena
    regrow (which rebuilds the graphs) and an overflowing step that is
    skipped and run again."""
    s = scenes.pyramid(layers=10)
    outs = []
    for graph, cap in ((0, 0), (1, 0), (1, 1)):
        gpu = backend_mod.GpuBackend(abi.default_params(**s.params, body_order=abi.ORDER_PRIORITY, graph=graph,
                                                        max_pairs_per_body=cap))
        gpu.pack(s.world())
        gpu.step(40)
        gpu.idle()
        st = gpu.last_stats
        assert st["overflow"] == 0 and st["steps"] == 40
        assert (st["graph_steps"] > 0) == (graph == 1)
        outs.append(gpu.read_state())
    for o in outs[1:]:
        assert np.array_equal(outs[0].pos, o.pos) and np.array_equal(outs[0].quat, o.quat)


def test_autotune_restores_state_and_keeps_parity(abi, scenes, backend_mod):
    """avbd_autotune times its candidate configurations from the current
    state and puts that state back exactly; the next step under the chosen
    configuration matches the oracle's step from the same state."""
    s = scenes.pyramid(layers=8)
    params, s0 = warm_state(abi, s, 30)
    gpu = backend_mod.GpuBackend(params)
    gpu.pack(s0)
    gpu.step(2)
    gpu.idle()
    before = gpu.read_state(manifolds=True)
    t = gpu.autotune(2)
    assert t["candidates"] >= 10 and t["best_ms"] <= t["default_ms"] and t["bodies"] == s0.n_bodies
    after = gpu.read_state(manifolds=True)
    assert np.array_equal(before.pos, after.pos) and np.array_equal(before.quat, after.quat)
    assert after.manifold_dict() == before.manifold_dict()
    assert np.array_equal(before.m_lambda[:before.m_count], after.m_lambda[:after.m_count])
    ref = Oracle(params, before.round_to_device())
    ref.step(1)
    gpu.step(1)
    gpu.idle()
    dyn = s0.mass > 0
    assert np.max(np.abs(gpu.read_state().pos[dyn] - ref.state().pos[dyn])) <= 1e-5


@pytest.mark.parametrize("schedule", [0, 1])
def test_uniform_grab_matches_oracle(abi, scenes, backend_mod, schedule):
    """The topology-free grab (backend.js:302-307, shaders.js:2119-2161)
    through avbd_set_grab, against the oracle's grab: one step from the same
    state within 1e-5 m, then 20 steps with the target moved before each step
    (as the app's pointer drag does, boot.js:633-636) within 5e-3 m, then a
    release; the grab changes no topology (same colouring as without it)."""
    s = scenes.cube_stack(n=6, beta=None)
    params = abi.default_params(**s.params, body_order=abi.ORDER_PRIORITY, schedule=schedule)
    o = Oracle(params, s.world())
    o.step(20)
    s0 = o.state().round_to_device()
    body, local = 4, np.array([0.3, -0.2, 0.5])
    k = max(400.0, 900.0 * s0.mass[body])
    target = s0.pos[body] + local + np.array([0.2, 0.1, 0.6])
    ref = Oracle(params, s0)
    gpu = backend_mod.GpuBackend(params)
    gpu.pack(s0)
    ref.set_grab(body, local, target, k)
    gpu.set_grab(body, local, target, k)
    ref.step(1)
    gpu.step(1)
    gpu.idle()
    dyn = s0.mass > 0
    want, got = ref.state(), gpu.read_state()
    assert np.max(np.abs(got.pos[dyn] - want.pos[dyn])) <= 1e-5
    assert np.max(np.abs(got.quat[dyn] - want.quat[dyn])) <= 1e-5
    assert np.array_equal(gpu.read_coloring()[0], ref.coloring()[0])
    for step in range(20):
        target = target + np.array([0.02, 0.0, 0.03])
        ref.set_grab(body, local, target, k)
        gpu.set_grab(body, local, target, k)
        ref.step(1)
        gpu.step(1)
    gpu.idle()
    want, got = ref.state(), gpu.read_state()
    assert want.pos[body, 2] > s0.pos[body, 2] + 0.5
    assert np.max(np.abs(got.pos[dyn] - want.pos[dyn])) < 5e-3
    ref.set_grab(-1)
    gpu.set_grab(-1)
    ref.step(3)
    gpu.step(3)
    gpu.idle()
    assert np.max(np.abs(gpu.read_state().pos[dyn] - ref.state().pos[dyn])) < 5e-3


def test_state_upload_round_trip_and_non_finite_rejection(abi, scenes, backend_mod):
    """avbd_write_state copies the caller's f64 arrays to the device as they
    are and converts them there: reading the state back gives the positions
    exactly and the f32-held fields rounded to f32. A position that is not
    finite is caught on the device: AVBD_ERR_NAN naming the first such body,
    and the device state stays what it was."""
    s = scenes.pyramid(layers=6)
    gpu = backend_mod.GpuBackend(abi.default_params(**s.params))
    gpu.pack(s.world())
    gpu.step(4)
    host = gpu.read_state()
    rng = np.random.default_rng(7)
    host.pos = host.pos + rng.normal(0.0, 1e-3, host.pos.shape)
    host.vel = rng.normal(0.0, 1.0, host.vel.shape)
    gpu.write_state(host)
    back = gpu.read_state()
    f32 = lambda a: a.astype(np.float32).astype(np.float64)
    assert np.array_equal(back.pos, host.pos)
    assert np.array_equal(back.vel, f32(host.vel))
    assert np.array_equal(back.quat, f32(host.quat))
    bad = host.copy()
    bad.pos[5, 1] = np.nan
    bad.pos[9, 0] = np.inf
    with pytest.raises(backend_mod.AvbdError) as e:
        gpu.write_state(bad)
    assert e.value.code == abi.AVBD_ERR_NAN and "body 5" in str(e.value)
    after = gpu.read_state()
    assert np.array_equal(after.pos, back.pos) and np.array_equal(after.vel, back.vel)
    gpu.step(1)
    gpu.idle()


@pytest.mark.parametrize("name", ["pyramid", "joint_clique"])
def test_tail_segment_rule_does_not_change_results(abi, scenes, backend_mod, name):
    """The colour-phase schedule's tail segment - automatic (tail_div 0: only
    for steps of at least 16 colours), forced (8) or off (-1) - orders the
    same body updates, so the states are bit-identical; the pyramid has a few
    colours a step, the joint clique 72."""
    s = scenes.pyramid(layers=8) if name == "pyramid" else scenes.joint_clique()
    states = []
    for td in (0, 8, -1):
        gpu = backend_mod.GpuBackend(abi.default_params(**s.params, body_order=abi.ORDER_PRIORITY, tail_div=td))
        gpu.pack(s.world())
        gpu.step(12)
        gpu.idle()
        states.append(gpu.read_state())
        gpu.destroy()
    for other in states[1:]:
        assert np.array_equal(other.pos, states[0].pos) and np.array_equal(other.quat, states[0].quat)
        assert np.array_equal(other.vel, states[0].vel)
