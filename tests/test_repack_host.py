"""Host side of a topology edit (World.edited, World.carry_from): the
reference semantics the device repack is checked against. Erasing bodies
drops exactly their joints and springs and renumbers the rest in order;
appended bodies bring their own constraints; the carried warm-start
manifolds are the old live ones between two survivors, renumbered; a
reordering of survivors carries none."""
import numpy as np

from oracle import Oracle


def test_erase_drops_incident_constraints_and_renumbers(scenes):
    s = scenes.heavy_chain(links=6, springs=6)
    w = s.world()
    keep = np.ones(w.n_bodies, bool)
    gone = 3
    keep[gone] = False
    extra = scenes.Scene("x")
    a = extra.box((1, 1, 1), 1.0, 0.5, (0, 0, 9))
    b = extra.box((1, 1, 1), 1.0, 0.5, (0, 0, 11))
    extra.joint(a, b, (0, 0, 0.5), (0, 0, -0.5))
    new, ob, oj, osp = w.edited(keep, extra.world())
    assert new.n_bodies == w.n_bodies + 1
    assert np.array_equal(ob[:w.n_bodies - 1], np.nonzero(keep)[0]) and np.all(ob[w.n_bodies - 1:] == -1)
    new_of = {int(o): i for i, o in enumerate(ob) if o >= 0}
    for j, o in enumerate(oj):
        if o < 0:
            continue
        assert w.j_body_b[o] != gone and w.j_body_a[o] != gone
        assert new.j_body_b[j] == new_of[int(w.j_body_b[o])]
        assert new.j_body_a[j] == (-1 if w.j_body_a[o] < 0 else new_of[int(w.j_body_a[o])])
    dropped = {int(j) for j in np.nonzero((w.j_body_a == gone) | (w.j_body_b == gone))[0]}
    assert set(range(w.n_joints)) - set(int(o) for o in oj if o >= 0) == dropped
    assert oj[-1] == -1 and new.j_body_a[-1] == w.n_bodies - 1 and new.j_body_b[-1] == w.n_bodies
    order = np.concatenate([new.j_order, new.s_order])
    assert sorted(order.tolist()) == list(range(len(order)))
    # survivors keep their relative force-list order
    old_rank = np.concatenate([w.j_order[oj[oj >= 0]], w.s_order[osp[osp >= 0]]])
    new_rank = np.concatenate([new.j_order[oj >= 0], new.s_order[osp >= 0]])
    assert np.array_equal(np.argsort(old_rank), np.argsort(new_rank))


def test_carried_manifolds_are_the_survivors_pairs(abi, scenes):
    s = scenes.random_pile(80, seed=4)
    p = abi.default_params(**s.params, body_order=abi.ORDER_PRIORITY)
    o = Oracle(p, s.world())
    o.step(40)
    before = o.state()
    keep = np.ones(before.n_bodies, bool)
    keep[3::5] = False
    keep[0] = True
    new, ob, oj, osp = before.edited(keep)
    carried = new.carry_from(before, ob, oj, osp)
    new_of = {int(x): i for i, x in enumerate(ob) if x >= 0}
    want = {(new_of[a], new_of[b]): v for (a, b), v in before.manifold_dict().items()
            if a in new_of and b in new_of and v[0] > 0}
    assert carried.manifold_dict() == want and len(want) > 0
    assert np.array_equal(carried.pos, before.pos[ob])
    o2 = Oracle(p, carried)
    o2.step(3)
    assert np.all(np.isfinite(o2.state().pos))
    # a reordering of survivors carries no contacts
    perm = np.arange(new.n_bodies)[::-1].astype(np.int32)
    assert new.carry_from(before, ob[perm]).m_count == 0
