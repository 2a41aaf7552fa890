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
