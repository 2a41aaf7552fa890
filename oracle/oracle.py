"""ORACLE wrapper - test infrastructure only, never part of the product path.

ctypes binding of `liborc.so`, the C++ f64 restatement of the reference CPU
engine (oracle/avbd_oracle.cpp). Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg use it, as the checker.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liborc.so")
LIB_TANGENT = os.path.join(HERE, "liborc_t.so")
SRC = os.path.join(HERE, "avbd_oracle.cpp")
HEADER = os.path.join(os.path.dirname(HERE), "include", "avbd_cuda.h")  # the structs it reads
FLAGS = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math"]


def _stale(lib: str) -> bool:
    return not os.path.exists(lib) or any(os.path.getmtime(lib) < os.path.getmtime(f) for f in (SRC, HEADER))


def build(force: bool = False) -> str:
    """Compile the oracle with the flags that keep it a faithful f64
    restatement: no FMA contraction, no fast-math."""
    if force or _stale(LIB):
        subprocess.check_call(FLAGS + ["-o", LIB, SRC])
    return LIB


def build_tangent(force: bool = False) -> str:
    """The tangent oracle: the same source with a forward-mode dual-number
    scalar (-DORC_TANGENT), whose values follow the f64 build's operations."""
    if force or _stale(LIB_TANGENT):
        subprocess.check_call(FLAGS + ["-DORC_TANGENT", "-o", LIB_TANGENT, SRC])
    return LIB_TANGENT


_lib = None
_lib_tangent = None


def _bind(L, tangent=False):
    vp = C.c_void_p
    L.orc_create.restype = vp
    L.orc_create.argtypes = [vp]
    L.orc_destroy.argtypes = [vp]
    for name in ("orc_load", "orc_read_state", "orc_set_params"):
        getattr(L, name).argtypes = [vp, vp]
    L.orc_step.argtypes = [vp, C.c_int32]
    L.orc_set_body_order.argtypes = [vp, vp, C.c_int32]
    L.orc_read_coloring.argtypes = [vp, vp, vp]
    L.orc_priority_coloring.argtypes = [vp, vp, vp]
    L.orc_index_coloring.argtypes = [vp, vp, vp]
    L.orc_read_pairs.argtypes = [vp, vp, vp, C.c_int64, vp]
    L.orc_stats.argtypes = [vp, vp]
    L.orc_num_forces.argtypes = [vp, vp, vp, vp]
    L.orc_read_joint.argtypes = [vp, C.c_int32, vp, vp, vp]
    L.orc_contact_normal_c.argtypes = [vp, vp, C.c_int64, vp]
    L.orc_set_grab.argtypes = [vp, C.c_int32, vp, vp, C.c_double]
    if tangent:
        L.orc_t_dims.restype = C.c_int
        L.orc_t_seed.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, C.c_int32]
        L.orc_t_read_pos.argtypes = [vp, vp, vp]
        L.orc_t_freeze.argtypes = [C.c_int32]
        return L
    L.orc_world_moment.argtypes = [vp, C.c_int32, C.c_int32, vp]
    L.orc_collide.argtypes = [vp, C.c_int32, C.c_int32, vp, vp, vp, vp]
    L.orc_collide.restype = C.c_int
    for name in ("orc_solve6",):
        getattr(L, name).argtypes = [vp] * 7
    for name in ("orc_quat_subtract", "orc_quat_integrate", "orc_quat_rotate"):
        getattr(L, name).argtypes = [vp, vp, vp]
    L.orc_orthonormal.argtypes = [vp, vp]
    L.orc_color_priority.argtypes = [C.c_uint32]
    L.orc_color_priority.restype = C.c_uint32
    return L


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = _bind(C.CDLL(LIB))
    return _lib


def lib_tangent():
    global _lib_tangent
    if _lib_tangent is None:
        build_tangent()
        _lib_tangent = _bind(C.CDLL(LIB_TANGENT), tangent=True)
    return _lib_tangent


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class Oracle:
    """One f64 CPU solver instance holding one scene."""

    _library = staticmethod(lib)

    def __init__(self, params, world=None):
        self.params = params
        self.L = self._library()
        self.h = self.L.orc_create(C.byref(params))
        self.world = None
        if world is not None:
            self.load(world)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_destroy(self.h)
            self.h = None

    def set_params(self, params):
        self.params = params
        self.L.orc_set_params(self.h, C.byref(params))

    def load(self, world):
        self.world = world.copy()
        self._wc = self.world.c()
        self.L.orc_load(self.h, C.byref(self._wc))

    def set_body_order(self, order):
        order = np.ascontiguousarray(order, np.int32)
        self.L.orc_set_body_order(self.h, _p(order), len(order))

    def step(self, n=1):
        self.L.orc_step(self.h, n)

    def set_grab(self, body, local=(0.0, 0.0, 0.0), target=(0.0, 0.0, 0.0), stiffness=0.0):
        """The WebGPU backend's uniform mouse grab (shaders.js:2119-2161);
        body < 0 releases it."""
        a = np.ascontiguousarray(local, np.float64)
        b = np.ascontiguousarray(target, np.float64)
        if self.L.orc_set_grab(self.h, int(body), _p(a), _p(b), float(stiffness)) != 0:
            raise ValueError("bad grab")

    def num_forces(self):
        j, s, m = C.c_int32(), C.c_int32(), C.c_int32()
        self.L.orc_num_forces(self.h, C.byref(j), C.byref(s), C.byref(m))
        return j.value, s.value, m.value

    def state(self):
        """A World copy holding the current state, including manifolds."""
        w = self.world.copy()
        _, _, m = self.num_forces()
        w.ensure_manifold_capacity(max(m, 1))
        wc = w.c()
        self.L.orc_read_state(self.h, C.byref(wc))
        w.m_count = wc.manifolds.count
        return w

    def coloring(self):
        n = self.world.n_bodies
        c = np.zeros(n, np.int32)
        k = C.c_int32()
        self.L.orc_read_coloring(self.h, _p(c), C.byref(k))
        return c, k.value

    def priority_coloring(self):
        n = self.world.n_bodies
        c = np.zeros(n, np.int32)
        k = C.c_int32()
        self.L.orc_priority_coloring(self.h, _p(c), C.byref(k))
        return c, k.value

    def index_coloring(self):
        n = self.world.n_bodies
        c = np.zeros(n, np.int32)
        k = C.c_int32()
        self.L.orc_index_coloring(self.h, _p(c), C.byref(k))
        return c, k.value

    def pairs(self):
        cnt = C.c_int64()
        self.L.orc_read_pairs(self.h, None, None, 0, C.byref(cnt))
        a = np.zeros(max(cnt.value, 1), np.int32)
        b = np.zeros(max(cnt.value, 1), np.int32)
        self.L.orc_read_pairs(self.h, _p(a), _p(b), cnt.value, C.byref(cnt))
        return a[:cnt.value], b[:cnt.value]

    def stats(self):
        import importlib
        abi = importlib.import_module("avbd-sandbox_gb300.abi")
        st = abi.Stats()
        self.L.orc_stats(self.h, C.byref(st))
        return st.as_dict()

    def contact_normal_c(self):
        """The normal row of every live contact's last evaluated constraint C."""
        cnt = C.c_int64()
        self.L.orc_contact_normal_c(self.h, None, 0, C.byref(cnt))
        out = np.zeros(max(cnt.value, 1))
        self.L.orc_contact_normal_c(self.h, _p(out), cnt.value, C.byref(cnt))
        return out[:cnt.value]

    def joint(self, jid):
        pl = np.zeros(3)
        la = np.zeros(3)
        br = C.c_int32()
        self.L.orc_read_joint(self.h, jid, _p(pl), _p(la), C.byref(br))
        return pl, la, bool(br.value)

    def world_moment(self, i, rotated=True):
        out = np.zeros(9)
        self.L.orc_world_moment(self.h, i, 1 if rotated else 0, _p(out))
        return out.reshape(3, 3)

    def collide(self, a, b):
        basis = np.zeros(9)
        feat = np.zeros(8, np.uint32)
        ra = np.zeros((8, 3))
        rb = np.zeros((8, 3))
        n = self.L.orc_collide(self.h, a, b, _p(basis), _p(feat), _p(ra), _p(rb))
        return n, basis, feat[:n], ra[:n], rb[:n]


def solve6(a_lin, a_ang, a_cross, b_lin, b_ang):
    f = lambda x: np.ascontiguousarray(x, np.float64).ravel()
    a_lin, a_ang, a_cross, b_lin, b_ang = map(f, (a_lin, a_ang, a_cross, b_lin, b_ang))
    x_lin, x_ang = np.zeros(3), np.zeros(3)
    lib().orc_solve6(_p(a_lin), _p(a_ang), _p(a_cross), _p(b_lin), _p(b_ang), _p(x_lin), _p(x_ang))
    return x_lin, x_ang


def quat_subtract(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    o = np.zeros(3)
    lib().orc_quat_subtract(_p(o), _p(a), _p(b))
    return o


def quat_integrate(q, dw):
    q, dw = np.asarray(q, float), np.asarray(dw, float)
    o = np.zeros(4)
    lib().orc_quat_integrate(_p(o), _p(q), _p(dw))
    return o


def quat_rotate(q, v):
    q, v = np.asarray(q, float), np.asarray(v, float)
    o = np.zeros(3)
    lib().orc_quat_rotate(_p(o), _p(q), _p(v))
    return o


def orthonormal(n):
    n = np.asarray(n, float)
    o = np.zeros(9)
    lib().orc_orthonormal(_p(o), _p(n))
    return o.reshape(3, 3)


def color_priority(i):
    return lib().orc_color_priority(i)


class TangentOracle(Oracle):
    """The tangent oracle: the f64 restatement carrying `dims` forward-mode
    directional derivatives through every operation of the step (values
    identical to Oracle's). Inputs get a direction with the seed_* calls after
    loading; positions() returns the positions and their derivatives along
    each direction: the exact derivative of the discrete step, which central
    differences only approximate."""

    _library = staticmethod(lib_tangent)

    @property
    def dims(self) -> int:
        return self.L.orc_t_dims()

    def _seed(self, what, index, comp, direction):
        if self.L.orc_t_seed(self.h, what, index, comp, direction) != 0:
            raise ValueError(f"bad seed ({what}, {index}, {comp}, {direction})")

    def seed_velocity(self, body, comp, direction):
        """Linear velocity component `comp` of `body` (and its previous velocity)."""
        self._seed(0, body, comp, direction)

    def seed_friction(self, body, direction):
        self._seed(1, body, 0, direction)

    def seed_penalty_max(self, direction):
        self._seed(2, 0, 0, direction)

    def seed_joint_stiffness(self, joint, direction):
        """The finite linear and angular stiffness of joint `joint`."""
        self._seed(3, joint, 0, direction)

    def seed(self, kind, index, comp, direction):
        """One seed in the C ABI's form (AVBD_SEED_* kind, index, comp,
        direction), as avbd_adjoint_forward takes them."""
        self._seed(kind, index, comp, direction)

    @staticmethod
    def freeze_geometry(mode: int):
        """Deny the narrow phase's geometry its tangents in every tangent
        oracle of the process (bit 0: contact bases, bit 1: body-local anchors;
        0 restores the exact derivative)."""
        lib_tangent().orc_t_freeze(mode)

    def positions(self):
        n = self.world.n_bodies
        pos = np.zeros((n, 3))
        tan = np.zeros((n, 3, self.dims))
        self.L.orc_t_read_pos(self.h, _p(pos), _p(tan))
        return pos, tan

