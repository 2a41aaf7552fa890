"""Writes the differentiable wall's reference gradients (run from the repo
root: `python tests/golden/make_c5_gradients.py`): its objective, its central
differences on the f64 oracle at the two steps of tests/c5_gradients.py, and
its exact derivative from the tangent oracle - the reference an adjoint's
gradient is checked against. Two files, one per primal body order:
c5_gradients.json (the reference engine's order, newest body first) and
c5_gradients_priority.json (the colour order of the integer-priority
colouring, the schedule of the CUDA backend and of its differentiable step)."""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.dirname(HERE)):
    if p not in sys.path:
        sys.path.insert(0, p)

import c5_gradients as c5  # noqa: E402

FILES = {None: "c5_gradients.json", "priority": "c5_gradients_priority.json"}


def compute(abi, scenes, order):
    th = c5.theta0(abi)
    return {"steps": c5.STEPS, "names": list(c5.NAMES), "theta": th.tolist(),
            "body_order": "reference" if order is None else "priority",
            "objective": c5.objective(abi, scenes, th, c5.STEPS, order),
            "differences": {repr(h): c5.central_differences(abi, scenes, th, c5.STEPS, h, order).tolist()
                            for h in c5.H},
            "tangent": c5.tangent_gradient(abi, scenes, th, c5.STEPS, order)[1].tolist()}


def main():
    abi, scenes = c5.modules()
    for key, name in FILES.items():
        out = compute(abi, scenes, None if key is None else abi.ORDER_PRIORITY)
        with open(os.path.join(HERE, name), "w") as f:
            json.dump(out, f, indent=1)
            f.write("\n")
        print(name, json.dumps(out))


if __name__ == "__main__":
    main()
