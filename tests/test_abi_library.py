"""The C-ABI library builds for sm_103a, loads, and exports every function
declared in include/avbd_cuda.h (no GPU needed); the host side's ctypes
view of a world."""
import ctypes
import importlib
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "avbd_cuda.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(avbd_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ("avbd_create", "avbd_pack", "avbd_step", "avbd_read_state", "avbd_write_state",
                     "avbd_read_coloring", "avbd_read_stats", "avbd_last_error", "avbd_destroy"):
        assert required in names


def test_library_exports_every_declared_symbol():
    build = importlib.import_module("avbd-sandbox_gb300.build")
    path = build.build()
    lib = ctypes.CDLL(path)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_create_without_gpu_fails_cleanly():
    """On a machine without a GPU the library must refuse, not fall back."""
    import torch

    if torch.cuda.is_available():
        return
    backend = importlib.import_module("avbd-sandbox_gb300.backend")
    try:
        backend.GpuBackend()
    except backend.AvbdError as e:
        assert e.code == -3  # AVBD_ERR_CUDA
    else:
        raise AssertionError("GpuBackend() succeeded without a GPU")


def test_default_params_match_reference(abi):
    backend = importlib.import_module("avbd-sandbox_gb300.backend")
    L = backend.load_library()
    p = abi.Params()
    L.avbd_default_params(ctypes.byref(p))
    # src/physics/solver.js:92-236
    assert (p.dt, p.gravity, p.iterations) == (1 / 60, -10.0, 10)
    assert (p.beta_lin, p.beta_ang, p.alpha, p.gamma) == (1e4, 100.0, 0.95, 0.999)
    assert (p.penalty_min, p.penalty_max, p.collision_margin, p.stick_threshold) == (1.0, 1e10, 0.01, 1e-5)
    assert (p.rotated_inertia, p.spring_stiffness_ramp, p.spring_geometric_stiffness,
            p.cached_contact_jacobians, p.post_stabilize) == (1, 0, 1, 1, 0)


def test_world_ctypes_view_is_cached_until_an_array_or_count_changes(abi, scenes):
    """World.c() keeps its ctypes view while the world's arrays are the same
    objects and its counts the same values (the per-step write_state /
    read_state calls reuse it); replacing an array or changing a count gives
    a fresh view with the new pointer or count."""
    w = scenes.pyramid(layers=4).world()
    a = w.c()
    assert w.c() is a
    b = w.c(with_manifolds=False)
    assert b is not a and w.c(with_manifolds=False) is b and w.c() is a
    w.pos[0, 0] += 1.0  # in place: the same buffer, the same view
    assert w.c() is a
    w.pos = w.pos.copy()
    c = w.c()
    assert c is not a
    assert ctypes.cast(c.bodies.pos, ctypes.c_void_p).value == w.pos.ctypes.data
    w.m_count = w.m_count + 1
    d = w.c()
    assert d is not c and d.manifolds.count == w.m_count
