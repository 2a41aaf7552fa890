"""Identity-preserving repack (avbd_repack) through the C ABI.

After a topology edit - bodies erased, bodies appended, the joints and
springs of erased bodies dropped - the live device state follows each
carried element to its new index, gathered on the device:

  * the device repack gives bit for bit the same following steps as the
    CPU handover of the same edit (read the state, apply the edit on the
    host with World.carry_from, pack), warm-start contacts included;
  * one step after the edit matches the oracle stepping the same edited
    state: pairs and manifold topology identical, positions within the
    FP32 single-step bound (1e-5 m);
  * broken joints and torn springs stay broken across the index shift;
  * survivors out of their old order carry no contacts (a fresh contact
    generation, as the reference starts then); bad maps are rejected.
"""
import importlib

import numpy as np
import pytest

from oracle import Oracle

pytestmark = pytest.mark.gpu
POS_TOL = 1e-5


@pytest.fixture(scope="module")
def backend_mod():
    return importlib.import_module("avbd-sandbox_gb300.backend")


def params_for(abi, s):
    return abi.default_params(**s.params, body_order=abi.ORDER_PRIORITY)


def extra_boxes(abi, scenes, n, z0):
    sc = scenes.Scene("extra")
    for k in range(n):
        sc.box((0.6, 0.6, 0.6), 500.0, 0.5, (0.7 * k - 1.0, 0.3, z0 + 0.8 * k))
    return sc.world()


def edit_of(abi, scenes, name):
    """(scene, steps before the edit, keep mask, appended world)"""
    if name == "pile":
        s = scenes.random_pile(200, seed=11)
        n = s.world().n_bodies
        keep = np.ones(n, bool)
        keep[5::7] = False
        keep[0] = True  # the ground
        return s, 40, keep, extra_boxes(abi, scenes, 3, 12.0)
    if name == "breakage":
        s = scenes.breakage()
        n = s.world().n_bodies
        keep = np.ones(n, bool)
        keep[2] = False  # a brick of the bottom row: every later index shifts
        return s, 10, keep, None
    if name == "chain":
        s = scenes.heavy_chain(links=8, springs=10)
        n = s.world().n_bodies
        keep = np.ones(n, bool)
        keep[n - 4] = False  # a point body in the spring chain
        return s, 15, keep, extra_boxes(abi, scenes, 2, 30.0)
    raise KeyError(name)


def states_equal(a, b):
    for f in ("pos", "quat", "vel", "omega", "prev_vel", "j_penalty_lin", "j_lambda_lin", "j_lambda_ang", "j_broken",
              "s_penalty", "s_peak_strain", "s_broken"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f
    assert a.m_count == b.m_count
    for f in ("m_body_a", "m_body_b", "m_num_contacts", "m_feature", "m_r_a", "m_penalty", "m_lambda", "m_stick"):
        assert np.array_equal(getattr(a, f)[:a.m_count], getattr(b, f)[:b.m_count]), f


@pytest.mark.parametrize("name", ["pile", "breakage", "chain"])
def test_device_repack_equals_host_handover(abi, scenes, backend_mod, name):
    s, k, keep, extra = edit_of(abi, scenes, name)
    p = params_for(abi, s)
    w0 = s.world()
    a, b = backend_mod.GpuBackend(p), backend_mod.GpuBackend(p)
    for g in (a, b):
        g.pack(w0)
        g.step(k)
        g.idle()
    before = b.read_state(manifolds=True)
    new, ob, oj, osp = before.edited(keep, extra)
    carried = a.repack(new, ob, oj, osp)
    host = new.carry_from(before, ob, oj, osp)
    assert carried == host.m_count
    if name != "chain":  # the chain's survivors share no contacts
        assert carried > 0
    b.pack(host)
    for g in (a, b):
        g.step(8)
        g.idle()
    states_equal(a.read_state(manifolds=True), b.read_state(manifolds=True))


@pytest.mark.parametrize("name", ["pile", "breakage", "chain"])
def test_edit_matches_the_oracle(abi, scenes, backend_mod, name):
    s, k, keep, extra = edit_of(abi, scenes, name)
    p = params_for(abi, s)
    gpu = backend_mod.GpuBackend(p)
    gpu.pack(s.world())
    gpu.step(k)
    gpu.idle()
    before = gpu.read_state(manifolds=True)
    new, ob, oj, osp = before.edited(keep, extra)
    gpu.repack(new, ob, oj, osp)
    ref = Oracle(p, new.carry_from(before, ob, oj, osp).round_to_device())
    gpu.step(1)
    gpu.idle()
    ref.step(1)
    got, want = gpu.read_state(manifolds=True), ref.state()
    ga, gb = gpu.read_pairs()
    oa, obb = ref.pairs()
    assert np.array_equal(ga, oa) and np.array_equal(gb, obb)
    assert got.manifold_dict() == want.manifold_dict()
    dyn = want.mass > 0
    assert np.max(np.abs(got.pos[dyn] - want.pos[dyn])) <= POS_TOL
    assert np.array_equal(got.j_broken, want.j_broken) and np.array_equal(got.s_broken, want.s_broken)


def test_broken_and_torn_survive_the_index_shift(abi, scenes, backend_mod):
    s, _, keep, _ = edit_of(abi, scenes, "breakage")
    gpu = backend_mod.GpuBackend(params_for(abi, s))
    gpu.pack(s.world())
    gpu.step(12)
    gpu.idle()
    before = gpu.read_state()
    assert before.j_broken.any() and before.s_broken.any()
    new, ob, oj, osp = before.edited(keep)
    gpu.repack(new, ob, oj, osp)
    after = gpu.read_state()
    assert np.array_equal(after.j_broken, before.j_broken[oj])
    assert np.array_equal(after.s_broken, before.s_broken[osp])
    assert np.array_equal(after.pos, before.pos[ob])


def test_reordered_survivors_start_a_fresh_contact_generation(abi, scenes, backend_mod):
    s = scenes.random_pile(60, seed=3)
    p = params_for(abi, s)
    gpu = backend_mod.GpuBackend(p)
    gpu.pack(s.world())
    gpu.step(30)
    gpu.idle()
    before = gpu.read_state(manifolds=True)
    n = before.n_bodies
    perm = np.concatenate([[0], np.arange(n - 1, 0, -1)]).astype(np.int32)  # ground first, the rest reversed
    new = before.edited(np.ones(n, bool))[0]
    for f in ("shape", "size", "mass", "moment", "radius", "friction", "pos", "quat", "vel", "omega", "prev_vel"):
        setattr(new, f, np.ascontiguousarray(getattr(before, f)[perm]))
    assert gpu.repack(new, perm) == 0
    host = new.carry_from(before, perm)
    assert host.m_count == 0
    ref = Oracle(p, host.round_to_device())
    gpu.step(1)
    gpu.idle()
    ref.step(1)
    got, want = gpu.read_state(manifolds=True), ref.state()
    assert got.manifold_dict() == want.manifold_dict()
    dyn = want.mass > 0
    assert np.max(np.abs(got.pos[dyn] - want.pos[dyn])) <= POS_TOL


def test_bad_maps_are_rejected(abi, scenes, backend_mod):
    s = scenes.cube_stack(n=4)
    gpu = backend_mod.GpuBackend(params_for(abi, s))
    w = s.world()
    gpu.pack(w)
    n = w.n_bodies
    for bad in (np.full(n, 0), np.full(n, n), np.full(n, -2)):
        with pytest.raises(backend_mod.AvbdError) as e:
            gpu.repack(w, bad)
        assert e.value.code == abi.AVBD_ERR_ARG
    with pytest.raises(ValueError):
        gpu.repack(w, np.arange(n - 1))
