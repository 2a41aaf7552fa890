"""The oracle's uniform mouse grab (the WebGPU backend's, src/physics/gpu/
shaders.js:2119-2161) against the CPU engine's drag joint (src/app/
boot.js:590-610: `new Joint(solver, null, body, world, local, stiffness, 0)`).
With gamma = 1 the drag joint's warm-started penalty equals its stiffness
(joint.js:150-157) and stays there (a finite joint ramps only up to its
stiffness and keeps no multiplier), so the two are the same force: the
trajectories agree to rounding while the grab lifts the body."""
import numpy as np

from oracle import Oracle


def test_grab_equals_drag_joint(abi, scenes):
    s = scenes.cube_stack(n=4, beta=None)
    w = s.world()
    body, local, k = 3, np.array([0.3, -0.2, 0.5]), 900.0 * w.mass[3]
    target = w.pos[body] + local + np.array([0.4, 0.0, 1.5])
    params = abi.default_params(**s.params, body_order=abi.ORDER_PRIORITY, gamma=1.0)
    grab = Oracle(params, w)
    grab.set_grab(body, local, target, k)
    dragw = w.copy()
    n = dragw.n_joints
    for f in ("j_body_a", "j_body_b", "j_r_a", "j_r_b", "j_stiffness_lin", "j_stiffness_ang", "j_fracture",
              "j_penalty_lin", "j_penalty_ang", "j_lambda_lin", "j_lambda_ang", "j_broken", "j_order"):
        a = getattr(dragw, f)
        setattr(dragw, f, np.zeros((n + 1,) + a.shape[1:], a.dtype))
    dragw.j_body_a[0], dragw.j_body_b[0] = -1, body
    dragw.j_r_a[0], dragw.j_r_b[0] = target, local
    dragw.j_stiffness_lin[0], dragw.j_stiffness_ang[0], dragw.j_fracture[0] = k, 0.0, np.inf
    dragw.j_penalty_lin[0] = k
    drag = Oracle(params, dragw)
    z0 = w.pos[body, 2]
    for _ in range(30):
        grab.step(1)
        drag.step(1)
    a, b = grab.state(), drag.state()
    dyn = w.mass > 0
    assert np.max(np.abs(a.pos[dyn] - b.pos[dyn])) < 1e-9
    assert a.pos[body, 2] > z0 + 0.5  # lifted toward the target
    grab.set_grab(-1)
    grab.step(5)
