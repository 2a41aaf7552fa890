"""The oracle's restatement of the WebGPU engine's contact extensions
(AVBD_CONTACT_MATERIALS; src/physics/gpu/shaders.js:1105-1366, 1772-1849,
2235-2260; src/physics/rigid.js:144-214), on the CPU.

  * at rest with the default materials the model reduces to the CPU engine's
    (the default rest offsets are the collision margin) - bit for bit;
  * restitution: the first contact step of an impact faster than the
    threshold gets the bias e (closing - toRest); the next step does not
    (the impact is not re-armed); below the threshold there is none;
  * every friction force lies in its cone: the static cone for a contact
    flagged static, the dynamic one otherwise;
  * a deeper rest offset rests deeper;
  * materials are validated as Rigid.setMaterial validates them.
"""
import numpy as np
import pytest

from oracle import Oracle


def resting_box(scenes, z=0.49, v=(0.0, 0.0, 0.0)):
    s = scenes.Scene("box")
    scenes.add_ground(s, 0.5)
    s.box((1, 1, 1), 1000, 0.5, (0, 0, z), v)
    return s


def test_defaults_at_rest_equal_the_cpu_model(abi, scenes):
    s = resting_box(scenes)
    traj = {}
    for model in (abi.CONTACT_CPU, abi.CONTACT_MATERIALS):
        o = Oracle(abi.default_params(gravity=-9.81, contact_model=model), s.world())
        z = []
        for _ in range(40):
            o.step(1)
            z.append(o.state().pos.copy())
        traj[model] = np.array(z)
    assert np.array_equal(traj[abi.CONTACT_CPU], traj[abi.CONTACT_MATERIALS])


@pytest.mark.parametrize("threshold, armed", [(1.0, True), (10.0, False)])
def test_restitution_is_armed_once(abi, scenes, threshold, armed):
    s = resting_box(scenes, z=0.53, v=(0.0, 0.0, -3.0))
    w = s.world()
    e = 0.6
    w.set_materials(restitution=[0.0, e])
    p = abi.default_params(gravity=-9.81, contact_model=abi.CONTACT_MATERIALS, restitution_threshold=threshold)
    o = Oracle(p, w)
    seen = []
    for _ in range(4):
        before = o.state()
        o.step(1)
        st = o.state()
        seen.append((before, st))
    first = next(k for k, (_, st) in enumerate(seen) if st.m_count and st.m_num_contacts[0] > 0)
    before, st = seen[first]
    n = st.m_num_contacts[0]
    bias = st.m_restitution_bias[0, :n]
    if armed:
        vn = before.vel[1, 2]  # the box's normal velocity at the step's start (the ground is static)
        closing = -vn * p.dt
        c0 = st.m_c0[0, :n, 0]
        np.testing.assert_allclose(bias, e * (closing - np.maximum(0.0, c0)), rtol=1e-12)
        assert np.all(bias > 0)
    else:
        assert np.all(bias == 0)
    _, nxt = seen[first + 1]
    assert np.all(nxt.m_restitution_bias[0, :nxt.m_num_contacts[0]] == 0)


@pytest.mark.parametrize("kind", ["pile", "drop", "spheres"])
def test_forces_stay_in_their_cones(abi, scenes, kind):
    s, mat = scenes.material_scene(kind)
    w = s.world()
    w.set_materials(**mat)
    o = Oracle(abi.default_params(**s.params, contact_model=abi.CONTACT_MATERIALS), w)
    sf, df = np.asarray(mat["static_friction"]), np.asarray(mat["dynamic_friction"])
    checked = 0
    for _ in range(60):
        o.step(1)
        st = o.state()
        for m in range(st.m_count):
            a, b = st.m_body_a[m], st.m_body_b[m]
            mus, mud = np.sqrt(sf[a] * sf[b]), np.sqrt(df[a] * df[b])
            for c in range(st.m_num_contacts[m]):
                lam = st.m_lambda[m, c]
                ft, fn = np.hypot(lam[1], lam[2]), abs(lam[0])
                mu = mus if st.m_stick[m, c] else mud
                assert lam[0] <= 0
                assert ft <= mu * fn * (1 + 1e-9) + 1e-9, (m, c, ft, mu * fn)
                checked += 1
    assert checked > 20


def test_deeper_rest_offset_rests_deeper(abi, scenes):
    z = {}
    for ro in (-0.005, -0.03):
        s = resting_box(scenes)
        w = s.world()
        w.set_materials(rest_offset=[-0.005, ro])
        o = Oracle(abi.default_params(gravity=-9.81, contact_model=abi.CONTACT_MATERIALS), w)
        o.step(240)
        z[ro] = o.state().pos[1, 2]
    assert z[-0.03] < z[-0.005] - 0.015


@pytest.mark.parametrize("kw", [dict(static_friction=[0.5, 0.2], dynamic_friction=[0.5, 0.3]),
                                dict(restitution=[0.0, 1.5]), dict(contact_offset=[0.0, -0.1]),
                                dict(static_friction=[0.5, np.nan])])
def test_materials_are_validated(scenes, kw):
    w = resting_box(scenes).world()
    with pytest.raises(ValueError):
        w.set_materials(**kw)


@pytest.mark.parametrize("gap, expect", [(0.004, 4), (0.009, 4), (0.012, 0)])
def test_speculative_contacts_within_the_skin(abi, scenes, gap, expect):
    """The pair's contact skin (the two contact offsets, 0.005 each by
    default) generates contacts at a positive separation below it, with C0
    on the normal = the gap minus the rest distance; the CPU engine's
    collider generates none at any positive separation."""
    s = scenes.Scene("hover")
    scenes.add_ground(s, 0.5)
    s.box((1, 1, 1), 1000, 0.5, (0, 0, 0.5 + gap))
    s.sphere(0.6, 1000, 0.5, (3.0, 0, 0.3 + gap))
    for model in (abi.CONTACT_CPU, abi.CONTACT_MATERIALS):
        o = Oracle(abi.default_params(gravity=0.0, contact_model=model), s.world())
        o.step(1)
        st = o.state()
        got = {(int(a), int(b)): int(n) for a, b, n in zip(st.m_body_a[:st.m_count], st.m_body_b[:st.m_count],
                                                           st.m_num_contacts[:st.m_count])}
        if model == abi.CONTACT_CPU or not expect:
            assert sum(got.values()) == 0
            continue
        assert got == {(1, 0): 4, (2, 0): 1}
        m = list(zip(st.m_body_a, st.m_body_b)).index((1, 0))
        np.testing.assert_allclose(st.m_c0[m, :4, 0], gap + 0.01, atol=1e-12)
