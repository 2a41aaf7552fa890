"""Element-wise comparison of the constraint state of two worlds (the device
against the oracle after the same step).

Per contact (manifolds matched by body pair, contacts by slot: the feature
IDs of the two sides are equal slot for slot): the multiplier lambda and the
penalty k of the normal and the two friction rows (manifold.js:447-491), the
stick flag, the warm-start anchors rA, rB and C0 (manifold.js:214-318). Per
joint: lambda and k of the linear and angular rows and the broken flag
(joint.js:255-317). Per spring: penalty, broken flag and peak strain
(spring.js:461-470, 618-634).

Errors are relative with a floor, |got - want| / max(|want|, floor), so that
values near zero are compared absolutely; the floor of each quantity is its
natural scale in these scenes (1 N for multipliers, 1 N/m for penalties,
1e-3 m for the body-local anchors, 1 m for C0 - so its error reads as
metres - and 1e-3 for strains).
"""
from __future__ import annotations

import numpy as np

FLOORS = {"lambda": 1.0, "penalty": 1.0, "r_a": 1e-3, "r_b": 1e-3, "c0": 1.0, "strain": 1e-3}


def rel_err(got, want, floor):
    got = np.asarray(got, float)
    want = np.asarray(want, float)
    if got.size == 0:
        return np.zeros(0)
    return np.abs(got - want) / np.maximum(np.abs(want), floor)


def summary(e):
    """max, 99.9th and 50th percentile, count."""
    if e.size == 0:
        return {"n": 0, "max": 0.0, "p999": 0.0, "p50": 0.0}
    return {"n": int(e.size), "max": float(e.max()), "p999": float(np.quantile(e, 0.999)),
            "p50": float(np.quantile(e, 0.5))}


def contact_arrays(w):
    """Live contacts of a world keyed for alignment: (A, B, slot) -> row index."""
    n = w.m_num_contacts[:w.m_count]
    rows = np.repeat(np.arange(w.m_count), n)
    slots = np.concatenate([np.arange(k) for k in n]) if len(n) else np.zeros(0, int)
    keys = (w.m_body_a[rows].astype(np.int64) << 36) | (w.m_body_b[rows].astype(np.int64) << 4) | slots
    return keys, rows, slots


def matched_contacts(got, want):
    """Row/slot indices of the contacts present on both sides, aligned, and the
    number present on one side only."""
    kg, rg, sg = contact_arrays(got)
    kw, rw, sw = contact_arrays(want)
    common, ig, iw = np.intersect1d(kg, kw, assume_unique=True, return_indices=True)
    unmatched = len(kg) + len(kw) - 2 * len(common)
    return (rg[ig], sg[ig]), (rw[iw], sw[iw]), unmatched


def contact_errors(got, want):
    (rg, sg), (rw, sw), unmatched = matched_contacts(got, want)
    out = {"unmatched": int(unmatched), "count": int(len(rg))}
    for name, floor in (("lambda", FLOORS["lambda"]), ("penalty", FLOORS["penalty"])):
        g = getattr(got, "m_" + ("lambda" if name == "lambda" else "penalty"))[rg, sg]
        w = getattr(want, "m_" + ("lambda" if name == "lambda" else "penalty"))[rw, sw]
        out[name + "_normal"] = summary(rel_err(g[:, 0], w[:, 0], floor))
        out[name + "_tangent"] = summary(rel_err(g[:, 1:], w[:, 1:], floor).ravel())
    for name in ("r_a", "r_b", "c0"):
        g = getattr(got, "m_" + name)[rg, sg]
        w = getattr(want, "m_" + name)[rw, sw]
        out[name] = summary(rel_err(g, w, FLOORS[name]).ravel())
    stick_g = got.m_stick[rg, sg] != 0
    stick_w = want.m_stick[rw, sw] != 0
    # the stick decision |C_t| < threshold of a contact inside the friction
    # cone; a contact without normal force (lambda_n = 0) has a cone of zero
    # width, where the decision rests on whether F_t is exactly zero: it is in
    # f64 for a contact with no tangential motion, and f32 rounding makes it
    # a few ulp instead - those are counted apart
    active = want.m_lambda[rw, sw][:, 0] < 0
    out["stick_mismatch"] = int(np.count_nonzero((stick_g != stick_w) & active))
    out["stick_mismatch_unloaded"] = int(np.count_nonzero((stick_g != stick_w) & ~active))
    out["stick_count"] = int(np.count_nonzero(stick_w))
    out["active"] = int(np.count_nonzero(active))
    return out


def joint_errors(got, want):
    out = {"count": int(want.n_joints)}
    for name in ("lambda_lin", "lambda_ang"):
        out[name] = summary(rel_err(getattr(got, "j_" + name), getattr(want, "j_" + name), FLOORS["lambda"]).ravel())
    for name in ("penalty_lin", "penalty_ang"):
        out[name] = summary(rel_err(getattr(got, "j_" + name), getattr(want, "j_" + name), FLOORS["penalty"]).ravel())
    out["broken_mismatch"] = int(np.count_nonzero((got.j_broken != 0) != (want.j_broken != 0)))
    out["broken"] = int(np.count_nonzero(want.j_broken))
    return out


def spring_errors(got, want):
    out = {"count": int(want.n_springs)}
    out["penalty"] = summary(rel_err(got.s_penalty, want.s_penalty, FLOORS["penalty"]))
    out["peak_strain"] = summary(rel_err(got.s_peak_strain, want.s_peak_strain, FLOORS["strain"]))
    out["broken_mismatch"] = int(np.count_nonzero((got.s_broken != 0) != (want.s_broken != 0)))
    out["broken"] = int(np.count_nonzero(want.s_broken))
    return out


def body_errors(got, want):
    dyn = want.mass > 0
    out = {}
    for name in ("pos", "quat", "vel", "omega"):
        d = np.abs(getattr(got, name)[dyn] - getattr(want, name)[dyn])
        out[name] = float(d.max()) if d.size else 0.0
    return out


def all_errors(got, want):
    return {"bodies": body_errors(got, want), "contacts": contact_errors(got, want),
            "joints": joint_errors(got, want), "springs": spring_errors(got, want)}


def scene_slice(w, s):
    """Scene `s` of a batched world as a world of its own (abi.World.scene)."""
    return w.scene(s)
