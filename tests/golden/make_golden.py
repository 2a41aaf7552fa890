"""Writes the golden fixtures of tests/test_golden.py (run from the repo root:
`python tests/golden/make_golden.py`).

Each fixture is one small scene advanced by the f64 oracle (the restatement of
the reference CPU engine in oracle/) for a few warm steps, its state rounded
to what the device stores, and the oracle's next step from it: candidate
pairs, manifolds (pairs, contact counts, feature IDs, anchors), colouring and
body state. The oracle replays the device's priority colouring
(ORDER_PRIORITY), so the device must reproduce the discrete outputs exactly
and the body state within the FP32 tolerances of the tests.
"""
import importlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

abi = importlib.import_module("avbd-sandbox_gb300.abi")
scene = importlib.import_module("avbd-sandbox_gb300.scene")


def cases():
    """name -> (scene, warm steps)"""
    return {
        "cube_stack": (scene.cube_stack(), 20),
        "pyramid6": (scene.pyramid(layers=6), 25),
        "heavy_chain8": (scene.heavy_chain(links=8, springs=10), 15),
        "spheres": (scene.spheres_scene(), 20),
        "brick_wall": (scene.brick_wall(cols=6, rows=4), 10),
        "pile": (scene.random_pile(60, seed=11), 60),
    }


def params_arrays(p):
    return {"p_" + name: np.asarray(getattr(p, name)) for name, _ in p._fields_}


def params_from_arrays(d):
    p = abi.Params()
    for name, ctype in p._fields_:
        v = d["p_" + name]
        setattr(p, name, float(v) if ctype in (abi.C.c_double, abi.C.c_float) else int(v))
    return p


def make(name, s, warm):
    from oracle import Oracle

    params = abi.default_params(**s.params, body_order=abi.ORDER_PRIORITY)
    o = Oracle(params, s.world())
    o.step(warm)
    inp = o.state().round_to_device()
    ref = Oracle(params, inp)
    ref.step(1)
    out = ref.state()
    a, b = ref.pairs()
    col, ncol = ref.coloring()
    d = {}
    d.update(params_arrays(params))
    d.update(inp.to_arrays("in_"))
    d.update(out.to_arrays("out_"))
    d["pairs_a"], d["pairs_b"] = a, b
    d["coloring"], d["num_colors"] = col, np.int64(ncol)
    d["warm_steps"] = np.int64(warm)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **d)
    return len(a), out.m_count


if __name__ == "__main__":
    for name, (s, warm) in cases().items():
        n_pairs, n_man = make(name, s, warm)
        print(f"{name}: {s.world().n_bodies} bodies, {n_pairs} pairs, {n_man} manifolds")
