"""ctypes mirror of include/avbd_cuda.h and numpy-backed world buffers.

`World` owns numpy arrays for every field of `avbd_world` and exposes a
ctypes struct whose pointers reference them, so the same object can be handed
to the CUDA backend (`libavbd_gb300.so`) and to the f64 oracle used by the
tests. Field order and types must match include/avbd_cuda.h exactly.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

AVBD_OK = 0
AVBD_ERR_ARG = -1
AVBD_ERR_CAPACITY = -2
AVBD_ERR_CUDA = -3
AVBD_ERR_TIMEOUT = -4
AVBD_ERR_NAN = -5
AVBD_ERR_STATE = -6

SHAPE_BOX = 0
SHAPE_SPHERE = 1

ORDER_REFERENCE = 0
ORDER_EXPLICIT = 1
ORDER_PRIORITY = 2
CONTACT_CPU = 0
CONTACT_MATERIALS = 1

MAX_CONTACTS = 8
MAX_COLORS = 1024

_d = C.POINTER(C.c_double)
_i = C.POINTER(C.c_int32)
_u = C.POINTER(C.c_uint32)


class Params(C.Structure):
    _fields_ = [
        ("dt", C.c_double), ("gravity", C.c_double),
        ("iterations", C.c_int32), ("post_stabilize", C.c_int32),
        ("beta_lin", C.c_double), ("beta_ang", C.c_double),
        ("alpha", C.c_double), ("gamma", C.c_double),
        ("penalty_min", C.c_double), ("penalty_max", C.c_double),
        ("collision_margin", C.c_double), ("stick_threshold", C.c_double),
        ("rotated_inertia", C.c_int32), ("spring_stiffness_ramp", C.c_int32),
        ("spring_geometric_stiffness", C.c_int32), ("cached_contact_jacobians", C.c_int32),
        ("broadphase", C.c_int32), ("hash_threshold", C.c_int32),
        ("body_order", C.c_int32), ("wait_limit", C.c_int32),
        ("fp64_ratio_threshold", C.c_double),
        ("max_pairs_per_body", C.c_int32), ("max_adjacency", C.c_int32),
        ("lanes_per_body", C.c_int32), ("blocks_per_sm", C.c_int32),
        ("schedule", C.c_int32), ("grid_factor", C.c_int32),
        ("neighbor_wait_limit", C.c_int32), ("tail_div", C.c_int32), ("graph", C.c_int32),
        ("contact_model", C.c_int32), ("contact_offset", C.c_double), ("rest_offset", C.c_double),
        ("restitution_threshold", C.c_double), ("contact_persistence", C.c_double),
    ]


def default_params(**overrides) -> Params:
    """`Solver.defaultParams()` (src/physics/solver.js:92-236)."""
    p = Params()
    p.dt = 1.0 / 60.0
    p.gravity = -10.0
    p.iterations = 10
    p.post_stabilize = 0
    p.beta_lin = 1e4
    p.beta_ang = 100.0
    p.alpha = 0.95
    p.gamma = 0.999
    p.penalty_min = 1.0
    p.penalty_max = 1e10
    p.collision_margin = 0.01
    p.stick_threshold = 1e-5
    p.rotated_inertia = 1
    p.spring_stiffness_ramp = 0
    p.spring_geometric_stiffness = 1
    p.cached_contact_jacobians = 1
    p.broadphase = 0
    p.hash_threshold = 150
    p.body_order = ORDER_REFERENCE
    p.fp64_ratio_threshold = 1e5
    p.schedule = 0
    p.contact_model = CONTACT_CPU
    p.contact_offset = 0.005
    p.rest_offset = -0.005
    p.restitution_threshold = 1.0
    p.contact_persistence = 0.002
    for k, v in overrides.items():
        if not hasattr(p, k):
            raise AttributeError(k)
        setattr(p, k, v)
    return p


class BodySoA(C.Structure):
    _fields_ = [("count", C.c_int32), ("shape", _i), ("size", _d), ("mass", _d), ("moment", _d),
                ("radius", _d), ("friction", _d), ("pos", _d), ("quat", _d), ("vel", _d),
                ("omega", _d), ("prev_vel", _d), ("static_friction", _d), ("dynamic_friction", _d),
                ("restitution", _d), ("contact_offset", _d), ("rest_offset", _d)]


class JointSoA(C.Structure):
    _fields_ = [("count", C.c_int32), ("body_a", _i), ("body_b", _i), ("r_a", _d), ("r_b", _d),
                ("stiffness_lin", _d), ("stiffness_ang", _d), ("fracture", _d),
                ("penalty_lin", _d), ("penalty_ang", _d), ("lambda_lin", _d), ("lambda_ang", _d),
                ("broken", _i), ("order", _i)]


class SpringSoA(C.Structure):
    _fields_ = [("count", C.c_int32), ("body_a", _i), ("body_b", _i), ("r_a", _d), ("r_b", _d),
                ("stiffness", _d), ("rest", _d), ("tear_strain", _d), ("penalty", _d),
                ("peak_strain", _d), ("broken", _i), ("order", _i)]


class ManifoldSoA(C.Structure):
    _fields_ = [("count", C.c_int32), ("capacity", C.c_int32), ("body_a", _i), ("body_b", _i),
                ("num_contacts", _i), ("basis", _d), ("friction", _d), ("feature", _u),
                ("r_a", _d), ("r_b", _d), ("c0", _d), ("penalty", _d), ("lambda_", _d),
                ("stick", _i), ("order", _i), ("restitution_bias", _d)]


class WorldC(C.Structure):
    _fields_ = [("bodies", BodySoA), ("joints", JointSoA), ("springs", SpringSoA),
                ("manifolds", ManifoldSoA), ("num_scenes", C.c_int32), ("scene_start", _i)]


class Stats(C.Structure):
    _fields_ = [("bodies", C.c_int64), ("manifolds", C.c_int64), ("contacts", C.c_int64),
                ("candidate_pairs", C.c_int64), ("joints_broken", C.c_int64),
                ("springs_broken", C.c_int64), ("colors", C.c_int32), ("fp64_bodies", C.c_int32),
                ("overflow", C.c_uint32), ("steps", C.c_int32),
                ("max_constraint_error", C.c_double), ("max_lambda", C.c_double),
                ("max_penalty", C.c_double), ("graph_steps", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Tuning(C.Structure):
    _fields_ = [("schedule", C.c_int32), ("lanes_per_body", C.c_int32), ("tail_div", C.c_int32),
                ("blocks_per_sm", C.c_int32), ("candidates", C.c_int32), ("trial_steps", C.c_int32),
                ("default_ms", C.c_double), ("best_ms", C.c_double), ("bodies", C.c_int64),
                ("manifolds", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


TANGENT_DIMS = 5
SEED_VELOCITY = 0
SEED_FRICTION = 1
SEED_PENALTY_MAX = 2
SEED_JOINT_STIFFNESS = 3


class TangentSeed(C.Structure):
    _fields_ = [("kind", C.c_int32), ("index", C.c_int32), ("comp", C.c_int32), ("dir", C.c_int32)]


class DeviceViews(C.Structure):
    _fields_ = [("body_pos", C.c_void_p), ("body_quat", C.c_void_p), ("body_count", C.c_int32),
                ("joint_state", C.c_void_p), ("joint_count", C.c_int32),
                ("spring_state", C.c_void_p), ("spring_count", C.c_int32)]


class Profile(C.Structure):
    _fields_ = [("broadphase_ms", C.c_double), ("narrowphase_ms", C.c_double),
                ("prepare_ms", C.c_double), ("coloring_ms", C.c_double),
                ("solve_ms", C.c_double), ("step_ms", C.c_double),
                ("candidate_pairs", C.c_int64), ("manifolds", C.c_int64), ("contacts", C.c_int64),
                ("colors", C.c_int32), ("fp64_bodies", C.c_int32),
                ("np_face", C.c_int32), ("np_edge", C.c_int32), ("np_exact", C.c_int32),
                ("lanes_per_body", C.c_int32), ("via_graph", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def _ptr(a: np.ndarray | None, kind):
    if a is None:
        return C.cast(None, kind)
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(kind)


class World:
    """numpy SoA of a world (one scene or a batch of scenes)."""

    BODY_F = ("size", "mass", "moment", "radius", "friction", "pos", "quat", "vel", "omega", "prev_vel")
    MATERIAL_F = ("static_friction", "dynamic_friction", "restitution", "contact_offset", "rest_offset")

    def set_materials(self, static_friction=None, dynamic_friction=None, restitution=None, contact_offset=None,
                      rest_offset=None):
        """Per-body contact materials of AVBD_CONTACT_MATERIALS
        (Rigid.setMaterial, src/physics/rigid.js:144-214): arrays of n
        values or scalars; None leaves that field at its default (static and
        dynamic friction: `friction`; restitution 0; offsets: the params').
        Checks as setMaterial does: values finite, friction, restitution and
        the contact offset non-negative, restitution <= 1, dynamic <= static
        friction."""
        n = self.n_bodies
        vals = {"static_friction": static_friction, "dynamic_friction": dynamic_friction,
                "restitution": restitution, "contact_offset": contact_offset, "rest_offset": rest_offset}
        for k, v in vals.items():
            if v is None:
                continue
            a = np.broadcast_to(np.asarray(v, np.float64), (n,)).copy()
            if not np.all(np.isfinite(a)):
                raise ValueError(f"{k} must be finite")
            if k != "rest_offset" and np.any(a < 0):
                raise ValueError(f"{k} must be non-negative")
            if k == "restitution" and np.any(a > 1):
                raise ValueError("restitution must be in [0, 1]")
            setattr(self, k, a)
        sf = self.static_friction if self.static_friction is not None else self.friction
        df = self.dynamic_friction if self.dynamic_friction is not None else self.friction
        if np.any(df > sf):
            raise ValueError("dynamicFriction must not exceed staticFriction")
        self._c = None

    def __init__(self, n_bodies: int, n_joints: int = 0, n_springs: int = 0, manifold_capacity: int = 0,
                 scene_start=None):
        n, j, s, m = n_bodies, n_joints, n_springs, manifold_capacity
        self.shape = np.zeros(n, np.int32)
        self.size = np.ones((n, 3))
        self.mass = np.zeros(n)
        self.moment = np.zeros((n, 3))
        self.radius = np.zeros(n)
        self.friction = np.zeros(n)
        self.pos = np.zeros((n, 3))
        self.quat = np.zeros((n, 4))
        self.quat[:, 3] = 1.0
        self.vel = np.zeros((n, 3))
        self.omega = np.zeros((n, 3))
        self.prev_vel = np.zeros((n, 3))
        # contact materials (AVBD_CONTACT_MATERIALS); None = the defaults
        self.static_friction = None
        self.dynamic_friction = None
        self.restitution = None
        self.contact_offset = None
        self.rest_offset = None
        # joints
        self.j_body_a = np.zeros(j, np.int32)
        self.j_body_b = np.zeros(j, np.int32)
        self.j_r_a = np.zeros((j, 3))
        self.j_r_b = np.zeros((j, 3))
        self.j_stiffness_lin = np.full(j, math.inf)
        self.j_stiffness_ang = np.zeros(j)
        self.j_fracture = np.full(j, math.inf)
        self.j_penalty_lin = np.zeros((j, 3))
        self.j_penalty_ang = np.zeros((j, 3))
        self.j_lambda_lin = np.zeros((j, 3))
        self.j_lambda_ang = np.zeros((j, 3))
        self.j_broken = np.zeros(j, np.int32)
        self.j_order = np.arange(j, dtype=np.int32)
        # springs
        self.s_body_a = np.zeros(s, np.int32)
        self.s_body_b = np.zeros(s, np.int32)
        self.s_r_a = np.zeros((s, 3))
        self.s_r_b = np.zeros((s, 3))
        self.s_stiffness = np.zeros(s)
        self.s_rest = np.zeros(s)
        self.s_tear_strain = np.full(s, math.inf)
        self.s_penalty = np.zeros(s)
        self.s_peak_strain = np.zeros(s)
        self.s_broken = np.zeros(s, np.int32)
        self.s_order = np.arange(j, j + s, dtype=np.int32)
        # manifolds
        self.m_count = 0
        self._alloc_manifolds(m)
        if scene_start is None:
            scene_start = [0, n]
        self.scene_start = np.asarray(scene_start, np.int32)
        self._c = None

    def _alloc_manifolds(self, m: int):
        K = MAX_CONTACTS
        self.m_capacity = m
        self.m_body_a = np.zeros(m, np.int32)
        self.m_body_b = np.zeros(m, np.int32)
        self.m_num_contacts = np.zeros(m, np.int32)
        self.m_basis = np.zeros((m, 9))
        self.m_friction = np.zeros(m)
        self.m_feature = np.zeros((m, K), np.uint32)
        self.m_r_a = np.zeros((m, K, 3))
        self.m_r_b = np.zeros((m, K, 3))
        self.m_c0 = np.zeros((m, K, 3))
        self.m_penalty = np.zeros((m, K, 3))
        self.m_lambda = np.zeros((m, K, 3))
        self.m_stick = np.zeros((m, K), np.int32)
        self.m_order = np.zeros(m, np.int32)
        self.m_restitution_bias = np.zeros((m, K))
        self._c = None

    def ensure_manifold_capacity(self, m: int):
        if m > self.m_capacity:
            self._alloc_manifolds(m)

    @property
    def n_bodies(self):
        return len(self.mass)

    @property
    def n_joints(self):
        return len(self.j_body_a)

    @property
    def n_springs(self):
        return len(self.s_body_a)

    @property
    def num_scenes(self):
        return len(self.scene_start) - 1

    def c(self, with_manifolds: bool = True) -> WorldC:
        """The ctypes view, cached per `with_manifolds` while every array
        attribute is the same array and every other attribute has the same
        value (an array replaced or a count changed rebuilds it; the cached
        pointers keep their arrays alive, so an array's id is not reused
        while cached)."""
        d = self.__dict__
        sig = tuple((k, id(v)) if isinstance(v, np.ndarray) else (k, v) for k, v in d.items() if k != "_c")
        cache = d.get("_c")
        if isinstance(cache, dict) and with_manifolds in cache and cache[with_manifolds][0] == sig:
            return cache[with_manifolds][1]
        w = WorldC()
        b = w.bodies
        b.count = self.n_bodies
        b.shape = _ptr(self.shape, _i)
        for f in self.BODY_F + self.MATERIAL_F:
            setattr(b, f, _ptr(getattr(self, f), _d))
        j = w.joints
        j.count = self.n_joints
        j.body_a, j.body_b = _ptr(self.j_body_a, _i), _ptr(self.j_body_b, _i)
        for f in ("r_a", "r_b", "stiffness_lin", "stiffness_ang", "fracture", "penalty_lin",
                  "penalty_ang", "lambda_lin", "lambda_ang"):
            setattr(j, f, _ptr(getattr(self, "j_" + f), _d))
        j.broken, j.order = _ptr(self.j_broken, _i), _ptr(self.j_order, _i)
        s = w.springs
        s.count = self.n_springs
        s.body_a, s.body_b = _ptr(self.s_body_a, _i), _ptr(self.s_body_b, _i)
        for f in ("r_a", "r_b", "stiffness", "rest", "tear_strain", "penalty", "peak_strain"):
            setattr(s, f, _ptr(getattr(self, "s_" + f), _d))
        s.broken, s.order = _ptr(self.s_broken, _i), _ptr(self.s_order, _i)
        m = w.manifolds
        m.count = self.m_count if with_manifolds else 0
        m.capacity = self.m_capacity if with_manifolds else 0
        if with_manifolds:
            m.body_a, m.body_b = _ptr(self.m_body_a, _i), _ptr(self.m_body_b, _i)
            m.num_contacts = _ptr(self.m_num_contacts, _i)
            m.basis, m.friction = _ptr(self.m_basis, _d), _ptr(self.m_friction, _d)
            m.feature = _ptr(self.m_feature, _u)
            m.r_a, m.r_b, m.c0 = _ptr(self.m_r_a, _d), _ptr(self.m_r_b, _d), _ptr(self.m_c0, _d)
            m.penalty, m.lambda_ = _ptr(self.m_penalty, _d), _ptr(self.m_lambda, _d)
            m.stick, m.order = _ptr(self.m_stick, _i), _ptr(self.m_order, _i)
            m.restitution_bias = _ptr(self.m_restitution_bias, _d)
        w.num_scenes = self.num_scenes
        w.scene_start = _ptr(self.scene_start, _i)
        if not isinstance(cache, dict):
            cache = {}
        cache[with_manifolds] = (sig, w)
        self._c = cache
        return w

    def copy(self) -> "World":
        import copy as _copy
        out = _copy.copy(self)
        for k, v in self.__dict__.items():
            if isinstance(v, np.ndarray):
                setattr(out, k, v.copy())
        out._c = None
        return out

    def round_to_device(self) -> "World":
        """A copy whose dynamic state is exactly representable on the device.

        The CUDA backend keeps positions in f64 and orientations, velocities,
        penalties, multipliers and contact anchors in f32. Feeding this copy to
        both the oracle and the device makes their inputs identical.
        """
        w = self.copy()
        f32 = lambda a: a.astype(np.float32).astype(np.float64)
        w.quat = f32(w.quat)
        w.vel = f32(w.vel)
        w.omega = f32(w.omega)
        w.prev_vel = f32(w.prev_vel)
        for k in ("j_penalty_lin", "j_penalty_ang", "s_penalty", "m_r_a", "m_r_b", "m_penalty",
                  "m_lambda", "m_restitution_bias"):
            setattr(w, k, f32(getattr(w, k)))
        return w

    def to_arrays(self, prefix: str = "") -> dict:
        """Every array of the world (and the live manifold count), for np.savez."""
        out = {prefix + k: (v[:self.m_count] if k.startswith("m_") else v)
               for k, v in self.__dict__.items() if isinstance(v, np.ndarray)}
        out[prefix + "m_count"] = np.int64(self.m_count)
        return out

    @classmethod
    def from_arrays(cls, d, prefix: str = "") -> "World":
        w = cls(0)
        for k in list(w.__dict__):
            if isinstance(w.__dict__[k], np.ndarray) and prefix + k in d:
                setattr(w, k, np.array(d[prefix + k]))
        w.m_count = int(d[prefix + "m_count"])
        w.m_capacity = len(w.m_body_a)
        # manifold fields added after the arrays were written: zeros of the right shape
        if w.m_restitution_bias.shape[0] != w.m_capacity:
            w.m_restitution_bias = np.zeros((w.m_capacity, MAX_CONTACTS))
        w._c = None
        return w

    def scene(self, s: int) -> "World":
        """Scene `s` of a batched world as a world of its own: its bodies
        renumbered from 0, its joints, springs and manifolds (constraints
        never cross scenes)."""
        b0, b1 = int(self.scene_start[s]), int(self.scene_start[s + 1])
        js = np.nonzero((self.j_body_b >= b0) & (self.j_body_b < b1))[0]
        ss = np.nonzero((self.s_body_b >= b0) & (self.s_body_b < b1))[0]
        ms = np.nonzero((self.m_body_a[:self.m_count] >= b0) & (self.m_body_a[:self.m_count] < b1))[0]
        out = World(b1 - b0, len(js), len(ss), max(len(ms), 1))
        for f in ("shape", "size", "mass", "moment", "radius", "friction", "pos", "quat", "vel", "omega",
                  "prev_vel"):
            setattr(out, f, np.ascontiguousarray(getattr(self, f)[b0:b1]))
        for f in self.MATERIAL_F:
            if getattr(self, f) is not None:
                setattr(out, f, np.ascontiguousarray(getattr(self, f)[b0:b1]))
        for f in ("j_r_a", "j_r_b", "j_stiffness_lin", "j_stiffness_ang", "j_fracture", "j_penalty_lin",
                  "j_penalty_ang", "j_lambda_lin", "j_lambda_ang", "j_broken"):
            setattr(out, f, np.ascontiguousarray(getattr(self, f)[js]))
        out.j_body_a = np.where(self.j_body_a[js] < 0, -1, self.j_body_a[js] - b0).astype(np.int32)
        out.j_body_b = (self.j_body_b[js] - b0).astype(np.int32)
        for f in ("s_r_a", "s_r_b", "s_stiffness", "s_rest", "s_tear_strain", "s_penalty", "s_peak_strain",
                  "s_broken"):
            setattr(out, f, np.ascontiguousarray(getattr(self, f)[ss]))
        out.s_body_a = (self.s_body_a[ss] - b0).astype(np.int32)
        out.s_body_b = (self.s_body_b[ss] - b0).astype(np.int32)
        order = np.argsort(np.concatenate([self.j_order[js], self.s_order[ss]]), kind="stable")
        rank = np.empty(len(order), np.int32)
        rank[order] = np.arange(len(order), dtype=np.int32)
        out.j_order, out.s_order = rank[:len(js)].copy(), rank[len(js):].copy()
        out.m_count = len(ms)
        for f in ("m_num_contacts", "m_basis", "m_friction", "m_feature", "m_r_a", "m_r_b", "m_c0", "m_penalty",
                  "m_lambda", "m_stick", "m_restitution_bias"):
            getattr(out, f)[:len(ms)] = getattr(self, f)[ms]
        out.m_body_a[:len(ms)] = self.m_body_a[ms] - b0
        out.m_body_b[:len(ms)] = self.m_body_b[ms] - b0
        out.m_order[:len(ms)] = np.arange(len(ms))
        return out

    def edited(self, keep, extra: "World | None" = None):
        """The scene graph after an edit: the bodies with keep[i] true, in
        their order, then the bodies of `extra` appended (with its joints and
        springs, renumbered); joints and springs touching an erased body are
        dropped, the rest keep their relative force-list order. Returns the
        new world (this world's current state for the survivors, no
        manifolds) and the maps new -> old index of bodies, joints and springs
        (-1 for appended elements), as avbd_repack takes them."""
        keep = np.asarray(keep, bool)
        n0 = int(keep.sum())
        ex = extra if extra is not None else World(0)
        new_of = np.full(self.n_bodies, -1, np.int64)
        new_of[keep] = np.arange(n0)
        jk = (new_of[self.j_body_b] >= 0) & ((self.j_body_a < 0) | (new_of[np.maximum(self.j_body_a, 0)] >= 0))
        sk = (new_of[self.s_body_a] >= 0) & (new_of[self.s_body_b] >= 0)
        nj, ns = int(jk.sum()) + ex.n_joints, int(sk.sum()) + ex.n_springs
        w = World(n0 + ex.n_bodies, nj, ns)
        for f in ("shape", "size", "mass", "moment", "radius", "friction", "pos", "quat", "vel", "omega",
                  "prev_vel"):
            getattr(w, f)[:n0] = getattr(self, f)[keep]
            getattr(w, f)[n0:] = getattr(ex, f)
        for f in self.MATERIAL_F:
            mine, theirs = getattr(self, f), getattr(ex, f)
            if mine is None and theirs is None:
                continue
            default = {"static_friction": "friction", "dynamic_friction": "friction"}.get(f)
            fill = lambda src, a, wd: (a if a is not None else (getattr(src, default) if default else
                                                               np.full(src.n_bodies, np.nan)))
            a = np.concatenate([fill(self, mine, self)[keep], fill(ex, theirs, ex)])
            if np.isnan(a).any():
                raise ValueError(f"{f}: set on one side of the edit only; give both worlds the field")
            setattr(w, f, a)
        jf = ("j_r_a", "j_r_b", "j_stiffness_lin", "j_stiffness_ang", "j_fracture", "j_penalty_lin", "j_penalty_ang",
              "j_lambda_lin", "j_lambda_ang", "j_broken")
        sf = ("s_r_a", "s_r_b", "s_stiffness", "s_rest", "s_tear_strain", "s_penalty", "s_peak_strain", "s_broken")
        j0, s0 = int(jk.sum()), int(sk.sum())
        for f in jf:
            getattr(w, f)[:j0] = getattr(self, f)[jk]
            getattr(w, f)[j0:] = getattr(ex, f)
        for f in sf:
            getattr(w, f)[:s0] = getattr(self, f)[sk]
            getattr(w, f)[s0:] = getattr(ex, f)
        ja = self.j_body_a[jk]
        w.j_body_a[:j0] = np.where(ja < 0, -1, new_of[np.maximum(ja, 0)])
        w.j_body_b[:j0] = new_of[self.j_body_b[jk]]
        w.j_body_a[j0:] = np.where(ex.j_body_a < 0, -1, ex.j_body_a + n0)
        w.j_body_b[j0:] = ex.j_body_b + n0
        w.s_body_a[:s0] = new_of[self.s_body_a[sk]]
        w.s_body_b[:s0] = new_of[self.s_body_b[sk]]
        w.s_body_a[s0:] = ex.s_body_a + n0
        w.s_body_b[s0:] = ex.s_body_b + n0
        # force-list order: survivors in their old order, then the appended
        # forces in theirs
        old_rank = np.concatenate([self.j_order[jk], self.s_order[sk]]).astype(np.int64)
        new_rank = np.concatenate([ex.j_order, ex.s_order]).astype(np.int64) + (old_rank.max() + 1 if len(old_rank)
                                                                              else 0)
        rank = np.concatenate([old_rank, new_rank])
        order = np.empty(len(rank), np.int32)
        order[np.argsort(rank, kind="stable")] = np.arange(len(rank), dtype=np.int32)
        w.j_order[:j0], w.s_order[:s0] = order[:j0], order[j0:j0 + s0]
        w.j_order[j0:], w.s_order[s0:] = order[j0 + s0:j0 + s0 + ex.n_joints], order[j0 + s0 + ex.n_joints:]
        old_body = np.concatenate([np.nonzero(keep)[0], np.full(ex.n_bodies, -1)]).astype(np.int32)
        old_joint = np.concatenate([np.nonzero(jk)[0], np.full(ex.n_joints, -1)]).astype(np.int32)
        old_spring = np.concatenate([np.nonzero(sk)[0], np.full(ex.n_springs, -1)]).astype(np.int32)
        return w, old_body, old_joint, old_spring

    def carry_from(self, old: "World", old_body=None, old_joint=None, old_spring=None) -> "World":
        """A copy of this (edited) world with the live state of the elements
        it carries from `old` (the state before the edit): what avbd_repack
        does on the device, on the host. old_body[i] is the old index of body
        i or -1 (likewise joints and springs; None carries nothing of that
        kind). Bodies keep position, orientation and velocities; joints their
        penalties, multipliers and broken flag; springs penalty, peak strain
        and torn flag. When the carried bodies keep their old relative order,
        old's live manifolds between two carried bodies are carried,
        renumbered (keeping the pair order); otherwise there are none."""
        w = self.copy()
        ob = None if old_body is None else np.asarray(old_body, np.int64)
        if ob is not None:
            k = ob >= 0
            for f in ("pos", "quat", "vel", "omega", "prev_vel"):
                getattr(w, f)[k] = getattr(old, f)[ob[k]]
        for m, prefix, fields in ((old_joint, "j_", ("penalty_lin", "penalty_ang", "lambda_lin", "lambda_ang",
                                                     "broken")),
                                  (old_spring, "s_", ("penalty", "peak_strain", "broken"))):
            if m is None:
                continue
            m = np.asarray(m, np.int64)
            k = m >= 0
            for f in fields:
                getattr(w, prefix + f)[k] = getattr(old, prefix + f)[m[k]]
        w.m_count = 0
        if ob is None:
            return w
        carried = ob[ob >= 0]
        if len(carried) == 0 or np.any(np.diff(carried) <= 0):
            return w
        new_of = np.full(old.n_bodies, -1, np.int64)
        new_of[carried] = np.nonzero(ob >= 0)[0]
        live = np.arange(old.m_count)
        live = live[(old.m_num_contacts[live] > 0) & (new_of[old.m_body_a[live]] >= 0)
                    & (new_of[old.m_body_b[live]] >= 0)]
        w._alloc_manifolds(max(len(live), 1))
        w.m_count = len(live)
        for f in ("m_num_contacts", "m_basis", "m_friction", "m_feature", "m_r_a", "m_r_b", "m_c0", "m_penalty",
                  "m_lambda", "m_stick", "m_restitution_bias"):
            getattr(w, f)[:len(live)] = getattr(old, f)[live]
        w.m_body_a[:len(live)] = new_of[old.m_body_a[live]]
        w.m_body_b[:len(live)] = new_of[old.m_body_b[live]]
        w.m_order[:len(live)] = np.arange(len(live))
        return w

    def manifold_dict(self):
        """Live manifolds keyed by (A, B) -> (num_contacts, features tuple)."""
        out = {}
        for m in range(self.m_count):
            n = int(self.m_num_contacts[m])
            out[(int(self.m_body_a[m]), int(self.m_body_b[m]))] = (
                n, tuple(int(x) for x in self.m_feature[m, :n]))
        return out
