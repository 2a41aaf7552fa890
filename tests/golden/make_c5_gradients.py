"""Writes tests/golden/c5_gradients.json (run from the repo root:
`python tests/golden/make_c5_gradients.py`): the differentiable wall's
objective, its central differences on the f64 oracle at the two steps of
tests/c5_gradients.py, and its exact derivative from the tangent oracle: the
reference of an adjoint's gradient."""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.dirname(HERE)):
    if p not in sys.path:
        sys.path.insert(0, p)

import c5_gradients as c5  # noqa: E402


def main():
    abi, scenes = c5.modules()
    th = c5.theta0(abi)
    out = {"steps": c5.STEPS, "names": list(c5.NAMES), "theta": th.tolist(),
           "objective": c5.objective(abi, scenes, th, c5.STEPS),
           "differences": {repr(h): c5.central_differences(abi, scenes, th, c5.STEPS, h).tolist() for h in c5.H},
           "tangent": c5.tangent_gradient(abi, scenes, th, c5.STEPS)[1].tolist()}
    with open(os.path.join(HERE, "c5_gradients.json"), "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
