"""Golden fixtures (tests/golden/*.npz, written by tests/golden/make_golden.py).

CPU: the oracle, rebuilt on this machine, reproduces every fixture bit for
bit (the restatement uses only IEEE-exact operations with contraction off, so
its results do not depend on the host). GPU: the CUDA backend, from the
fixture's input state, reproduces the discrete outputs exactly and the body
state within the FP32 single-step tolerances.
"""
import glob
import importlib
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))
NAMES = [os.path.splitext(os.path.basename(f))[0] for f in FIXTURES]


def load(name):
    abi = importlib.import_module("avbd-sandbox_gb300.abi")
    d = np.load(os.path.join(HERE, "golden", name + ".npz"))
    p = abi.Params()
    for field, ctype in p._fields_:
        if "p_" + field not in d:  # a field added after the fixture was written keeps its zero default
            continue
        v = d["p_" + field]
        setattr(p, field, float(v) if ctype in (abi.C.c_double, abi.C.c_float) else int(v))
    return p, abi.World.from_arrays(d, "in_"), abi.World.from_arrays(d, "out_"), d


def test_fixtures_present():
    assert len(FIXTURES) >= 6


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_golden(name):
    from oracle import Oracle

    p, inp, out, d = load(name)
    o = Oracle(p, inp)
    o.step(1)
    got = o.state()
    for k in ("pos", "quat", "vel", "omega"):
        assert np.array_equal(getattr(got, k), getattr(out, k)), k
    a, b = o.pairs()
    assert np.array_equal(a, d["pairs_a"]) and np.array_equal(b, d["pairs_b"])
    assert got.manifold_dict() == out.manifold_dict()
    col, n = o.coloring()
    assert n == int(d["num_colors"]) and np.array_equal(col, d["coloring"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_cuda_matches_golden(name):
    backend = importlib.import_module("avbd-sandbox_gb300.backend")
    p, inp, out, d = load(name)
    gpu = backend.GpuBackend(p)
    gpu.pack(inp)
    gpu.step(1)
    gpu.idle()
    ga, gb = gpu.read_pairs()
    assert np.array_equal(ga, d["pairs_a"]) and np.array_equal(gb, d["pairs_b"]), "candidate pairs"
    got = gpu.read_state(manifolds=True)
    assert got.manifold_dict() == out.manifold_dict(), "manifold topology"
    col, n = gpu.read_coloring()
    assert n == int(d["num_colors"]) and np.array_equal(col, d["coloring"]), "colouring"
    dyn = out.mass > 0
    assert np.max(np.abs(got.pos[dyn] - out.pos[dyn])) <= 1e-5
    assert np.max(np.abs(got.quat[dyn] - out.quat[dyn])) <= 1e-5
    assert np.max(np.abs(got.vel[dyn] - out.vel[dyn])) <= 1e-3
