"""The WebGPU engine's contact extensions (AVBD_CONTACT_MATERIALS) on the
device against the oracle's restatement of them, through the C ABI.

Scenes with seeded per-body materials (static and dynamic friction,
restitution, rest offsets; scene.material_scene), stepped on the oracle to
a state, then one step on each side from that state (rounded to what the
device stores, warm-start manifolds and restitution biases included):
candidate pairs, manifold topology and colouring identical; body state and
every contact's multiplier, penalty, stick flag, anchors and C0 within the
dual-state bounds of tests/test_gpu_dual_state.py; every contact's
restitution bias within 1e-6 m + 1e-4 of its value (f32 velocities on the
device). The warm steps include impact steps, where biases are armed, and
the "hover" scene starts with bodies inside each other's contact skin
(speculative contacts at a positive separation).
"""
import importlib

import numpy as np
import pytest

import dual_state as ds
from oracle import Oracle
from test_gpu_dual_state import check_dual, check_discrete

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def backend_mod():
    return importlib.import_module("avbd-sandbox_gb300.backend")


def setup(abi, scenes, kind):
    s, mat = scenes.material_scene(kind)
    w = s.world()
    w.set_materials(**mat)
    p = abi.default_params(**s.params, body_order=abi.ORDER_PRIORITY, contact_model=abi.CONTACT_MATERIALS)
    return s, w, p


CASES = [("drop", 4), ("drop", 5), ("drop", 9), ("drop", 12), ("drop", 20), ("pile", 0), ("pile", 27), ("pile", 40),
         ("spheres", 0), ("spheres", 3), ("spheres", 11), ("spheres", 25), ("hover", 0), ("hover", 1), ("hover", 6)]


@pytest.mark.parametrize("kind, warm", CASES)
def test_materials_single_step(abi, scenes, backend_mod, kind, warm):
    s, w, p = setup(abi, scenes, kind)
    o = Oracle(p, w)
    o.step(warm)
    state = o.state().round_to_device()
    ref = Oracle(p, state)
    gpu = backend_mod.GpuBackend(p)
    gpu.pack(state)
    ref.step(1)
    gpu.step(1)
    gpu.idle()
    want, got = ref.state(), gpu.read_state(manifolds=True)
    check_discrete(ref, gpu, want, got)
    check_dual(got, want)
    (rg, sg), (rw, sw), _ = ds.matched_contacts(got, want)
    bg, bw = got.m_restitution_bias[rg, sg], want.m_restitution_bias[rw, sw]
    assert np.all(np.abs(bg - bw) <= 1e-6 + 1e-4 * np.abs(bw)), np.max(np.abs(bg - bw))


def test_biases_are_armed_on_the_device(abi, scenes, backend_mod):
    """The device arms restitution on its own trajectory (impacts of the drop
    scene) and the multiplier state stays finite."""
    s, w, p = setup(abi, scenes, "drop")
    gpu = backend_mod.GpuBackend(p)
    gpu.pack(w)
    armed = 0
    for _ in range(20):
        gpu.step(1)
        st = gpu.read_state(manifolds=True)
        armed += int(np.count_nonzero(st.m_restitution_bias[:st.m_count] > 0))
        assert np.all(np.isfinite(st.pos))
    assert armed > 0


def test_cpu_model_ignores_materials(abi, scenes, backend_mod):
    """Materials given to a context of the CPU contact model change nothing."""
    s, w, p = setup(abi, scenes, "drop")
    cpu = abi.default_params(**s.params, body_order=abi.ORDER_PRIORITY)
    a, b = backend_mod.GpuBackend(cpu), backend_mod.GpuBackend(cpu)
    a.pack(w)
    b.pack(s.world())
    a.step(10)
    b.step(10)
    a.idle()
    b.idle()
    assert np.array_equal(a.read_state().pos, b.read_state().pos)


def test_differentiable_step_rejects_the_materials_model(abi, scenes, backend_mod):
    s, w, p = setup(abi, scenes, "drop")
    gpu = backend_mod.GpuBackend(p)
    with pytest.raises(backend_mod.AvbdError) as e:
        gpu.adjoint_forward(w, 1, [])
    assert e.value.code == abi.AVBD_ERR_ARG
