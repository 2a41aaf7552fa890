"""Host-side mirror of the reference `GpuBackend` (src/physics/gpu/backend.js:243),
bound to the CUDA library through its C ABI (include/avbd_cuda.h).

Method names follow the reference so its call sites read the same:
  pack(world)          backend.js:662   topology + state upload
  step(n)              backend.js:1393  asynchronous device step(s)
  idle()               backend.js:1804  wait; raise on device-side errors
  read_state()         backend.js:2154  body/joint/spring (+ manifold) state
  sync_to_cpu(world)   backend.js:1984  write device state into a host world
  write_state(world)   CPU-authoritative handover back to the device
  read_coloring()      backend.js:2053
  last_stats           backend.js:309
  set_profiling(on) / last_profile      backend.js:1836-1897

There is no CPU fallback: when the CUDA library is missing or no GPU is
present, construction raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libavbd_gb300.so")

_lib = None


def load_library(path: str = LIB_PATH):
    """dlopen the CUDA backend. Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"CUDA extension not built: {path} is missing (run __graft_entry__.build())")
    L = C.CDLL(path)
    vp = C.c_void_p
    L.avbd_default_params.argtypes = [vp]
    L.avbd_default_params.restype = None
    L.avbd_create.argtypes = [vp, C.POINTER(vp)]
    L.avbd_destroy.argtypes = [vp]
    for name in ("avbd_pack", "avbd_read_state", "avbd_write_state", "avbd_read_stats", "avbd_read_profile",
                 "avbd_kernel_launches"):
        getattr(L, name).argtypes = [vp, vp]
    L.avbd_step.argtypes = [vp, C.c_int32]
    L.avbd_synchronize.argtypes = [vp]
    L.avbd_set_profiling.argtypes = [vp, C.c_int32]
    L.avbd_read_coloring.argtypes = [vp, vp, vp]
    L.avbd_read_pairs.argtypes = [vp, vp, vp, C.c_int64, vp]
    L.avbd_last_error.argtypes = [vp]
    L.avbd_last_error.restype = C.c_char_p
    L.avbd_overlap_pairs_static.argtypes = [C.c_int32, vp, vp, vp, C.c_double, vp, C.c_int64, vp, vp]
    L.avbd_overlap_pairs_static.restype = C.c_int
    L.avbd_set_coloring.argtypes = [vp, vp]
    L.avbd_set_coloring.restype = C.c_int
    L.avbd_update_joint_anchor.argtypes = [vp, C.c_int32, vp]
    L.avbd_update_joint_anchor.restype = C.c_int
    L.avbd_device_views_get.argtypes = [vp, vp]
    L.avbd_device_views_get.restype = C.c_int
    L.avbd_autotune.argtypes = [vp, C.c_int32, vp]
    L.avbd_autotune.restype = C.c_int
    L.avbd_set_grab.argtypes = [vp, C.c_int32, vp, vp, C.c_double]
    L.avbd_set_grab.restype = C.c_int
    L.avbd_repack.argtypes = [vp, vp, vp, vp, vp, vp]
    L.avbd_repack.restype = C.c_int
    L.avbd_adjoint_forward.argtypes = [vp, vp, C.c_int32, vp, C.c_int32]
    L.avbd_adjoint_read.argtypes = [vp, vp, vp, vp]
    L.avbd_adjoint_backward.argtypes = [vp, vp, vp]
    for name in ("avbd_adjoint_forward", "avbd_adjoint_read", "avbd_adjoint_backward"):
        getattr(L, name).restype = C.c_int
    for name in ("avbd_create", "avbd_destroy", "avbd_pack", "avbd_step", "avbd_synchronize", "avbd_read_state",
                 "avbd_write_state", "avbd_read_coloring", "avbd_read_pairs", "avbd_read_stats",
                 "avbd_set_profiling", "avbd_read_profile", "avbd_kernel_launches"):
        getattr(L, name).restype = C.c_int
    _lib = L
    return L


class AvbdError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"avbd error {code}: {msg}")
        self.code = code


class GpuBackend:
    def __init__(self, params: abi.Params | None = None, **overrides):
        self.L = load_library()
        if params is None:
            params = abi.Params()
            self.L.avbd_default_params(C.byref(params))
        for k, v in overrides.items():
            setattr(params, k, v)
        self.params = params
        h = C.c_void_p()
        rc = self.L.avbd_create(C.byref(params), C.byref(h))
        if rc != abi.AVBD_OK:
            raise AvbdError(rc, self.L.avbd_last_error(None).decode())
        self.h = h
        self.world = None

    def _check(self, rc):
        if rc != abi.AVBD_OK:
            raise AvbdError(rc, self.L.avbd_last_error(self.h).decode())

    def destroy(self):
        if getattr(self, "h", None):
            self.L.avbd_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    # --- reference interface -------------------------------------------------
    def pack(self, world: abi.World):
        self.world = world.copy()
        wc = self.world.c()
        self._check(self.L.avbd_pack(self.h, C.byref(wc)))

    def repack(self, world: abi.World, old_body=None, old_joint=None, old_spring=None) -> int:
        """avbd_repack: `world` is the edited scene graph; old_body[i] is the
        index new body i had before (-1: new), likewise for joints and springs
        (None: none carried). Carried elements keep their live device state;
        returns the number of warm-start manifolds carried."""
        maps = []
        for m, count in ((old_body, world.n_bodies), (old_joint, world.n_joints), (old_spring, world.n_springs)):
            if m is None:
                maps.append(None)
                continue
            a = np.ascontiguousarray(m, dtype=np.int32)
            if a.shape != (count,):
                raise ValueError(f"map of {a.shape} entries for {count} elements")
            maps.append(a)
        self.world = world.copy()
        wc = self.world.c(with_manifolds=False)
        carried = C.c_int64(0)
        ptr = [None if m is None else m.ctypes.data_as(C.c_void_p) for m in maps]
        self._check(self.L.avbd_repack(self.h, C.byref(wc), ptr[0], ptr[1], ptr[2], C.byref(carried)))
        return int(carried.value)

    def step(self, n: int = 1):
        self._check(self.L.avbd_step(self.h, n))

    def idle(self):
        self._check(self.L.avbd_synchronize(self.h))

    def read_state(self, manifolds: bool = False) -> abi.World:
        w = self.world.copy()
        if manifolds:
            st = self.last_stats
            w.ensure_manifold_capacity(max(int(st["manifolds"]), 1))
        wc = w.c(with_manifolds=manifolds)
        self._check(self.L.avbd_read_state(self.h, C.byref(wc)))
        w.m_count = wc.manifolds.count if manifolds else 0
        return w

    def sync_to_cpu(self, world: abi.World):
        wc = world.c(with_manifolds=False)
        self._check(self.L.avbd_read_state(self.h, C.byref(wc)))

    def write_state(self, world: abi.World):
        wc = world.c()
        self._check(self.L.avbd_write_state(self.h, C.byref(wc)))

    def read_coloring(self):
        n = self.world.n_bodies
        c = np.zeros(n, np.int32)
        k = C.c_int32()
        self._check(self.L.avbd_read_coloring(self.h, c.ctypes.data_as(C.c_void_p), C.byref(k)))
        return c, k.value

    def read_pairs(self):
        cnt = C.c_int64()
        self._check(self.L.avbd_read_pairs(self.h, None, None, 0, C.byref(cnt)))
        a = np.zeros(max(cnt.value, 1), np.int32)
        b = np.zeros(max(cnt.value, 1), np.int32)
        self._check(self.L.avbd_read_pairs(self.h, a.ctypes.data_as(C.c_void_p), b.ctypes.data_as(C.c_void_p),
                                           cnt.value, C.byref(cnt)))
        return a[:cnt.value], b[:cnt.value]

    def set_coloring(self, color_of):
        """uploadColoring / overrideColoring (backend.js:1925): colours to use
        from the next step on; None returns to the device's own colouring."""
        if color_of is None:
            self._check(self.L.avbd_set_coloring(self.h, None))
            return
        c = np.ascontiguousarray(color_of, dtype=np.int32)
        assert c.shape == (self.world.n_bodies,)
        self._check(self.L.avbd_set_coloring(self.h, c.ctypes.data_as(C.c_void_p)))

    def update_joint_anchor(self, joint: int, r_a):
        """updateJointAnchor (backend.js:1970-1978): joint's anchor on body A
        (a world point when the joint has no body A)."""
        a = np.ascontiguousarray(r_a, dtype=np.float64)
        self._check(self.L.avbd_update_joint_anchor(self.h, int(joint), a.ctypes.data_as(C.c_void_p)))

    def set_grab(self, body: int, local=(0.0, 0.0, 0.0), target=(0.0, 0.0, 0.0), stiffness: float = 0.0):
        """The reference's `grab` ({body, local, target, stiffness},
        backend.js:302-307): a topology-free pull of `body`'s local point
        toward the world `target`; body = -1 releases."""
        if body < 0:
            self._check(self.L.avbd_set_grab(self.h, -1, None, None, 0.0))
            return
        a = np.ascontiguousarray(local, dtype=np.float64)
        b = np.ascontiguousarray(target, dtype=np.float64)
        self._check(self.L.avbd_set_grab(self.h, int(body), a.ctypes.data_as(C.c_void_p),
                                         b.ctypes.data_as(C.c_void_p), float(stiffness)))

    def device_views(self) -> dict:
        """getConstraintGpuState (backend.js:1950-1967): device pointers of the
        live body poses and joint/spring state."""
        v = abi.DeviceViews()
        self._check(self.L.avbd_device_views_get(self.h, C.byref(v)))
        return {k: getattr(v, k) for k, _ in v._fields_}

    def autotune(self, trial_steps: int = 3) -> dict:
        """Time the solve's launch configurations from the current state, keep
        the fastest (the state is put back unchanged) and return the choice."""
        t = abi.Tuning()
        self._check(self.L.avbd_autotune(self.h, int(trial_steps), C.byref(t)))
        return t.as_dict()

    # --- the differentiable step ---------------------------------------------
    def adjoint_forward(self, world: abi.World, steps: int, seeds):
        """avbd_adjoint_forward: `steps` differentiable steps of `world`,
        seeds = [(kind, index, comp, direction), ...] (abi.SEED_*)."""
        arr = (abi.TangentSeed * max(len(seeds), 1))()
        for k, (kind, index, comp, d) in enumerate(seeds):
            arr[k] = abi.TangentSeed(kind, index, comp, d)
        self._tangent_world = world.copy()
        wc = self._tangent_world.c(with_manifolds=False)
        self._check(self.L.avbd_adjoint_forward(self.h, C.byref(wc), int(steps), arr, len(seeds)))

    def adjoint_read(self):
        """Positions (n, 3), their derivatives (n, 3, TANGENT_DIMS), orientations (n, 4)."""
        n = self._tangent_world.n_bodies
        pos = np.zeros((n, 3))
        dpos = np.zeros((n, 3, abi.TANGENT_DIMS))
        quat = np.zeros((n, 4))
        self._check(self.L.avbd_adjoint_read(self.h, pos.ctypes.data_as(C.c_void_p), dpos.ctypes.data_as(C.c_void_p),
                                             quat.ctypes.data_as(C.c_void_p)))
        return pos, dpos, quat

    def adjoint_backward(self, grad_pos) -> np.ndarray:
        """Vector-Jacobian product: d<grad_pos, pos_T> / d theta for each direction."""
        g = np.ascontiguousarray(grad_pos, dtype=np.float64)
        out = np.zeros(abi.TANGENT_DIMS)
        self._check(self.L.avbd_adjoint_backward(self.h, g.ctypes.data_as(C.c_void_p), out.ctypes.data_as(C.c_void_p)))
        return out

    @property
    def last_stats(self) -> dict:
        st = abi.Stats()
        self._check(self.L.avbd_read_stats(self.h, C.byref(st)))
        return st.as_dict()

    def set_profiling(self, on: bool):
        self._check(self.L.avbd_set_profiling(self.h, 1 if on else 0))

    @property
    def last_profile(self) -> dict:
        p = abi.Profile()
        self._check(self.L.avbd_read_profile(self.h, C.byref(p)))
        return p.as_dict()

    @property
    def kernel_launches(self) -> int:
        v = C.c_int64()
        self._check(self.L.avbd_kernel_launches(self.h, C.byref(v)))
        return v.value


STATIC_PAIRS_MAX_BODIES = 65000


def overlap_pairs_static(n, pos, radius, dynamic, cell_size, keys, capacity, count, stream=0):
    """avbd_overlap_pairs_static on device pointers (ints): the allocation-free
    bounding-sphere overlap query. Results are ready when `stream` reaches the
    end of the call; raises AvbdError on a rejected call."""
    L = load_library()
    rc = L.avbd_overlap_pairs_static(n, pos, radius, dynamic or None, cell_size, keys, capacity, count,
                                     stream or None)
    if rc != abi.AVBD_OK:
        raise AvbdError(rc, L.avbd_last_error(None).decode())
