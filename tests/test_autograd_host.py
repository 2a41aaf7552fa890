"""The torch.autograd.Function wrapper of the differentiable step, on the
host: a stand-in backend whose "run" is a known linear map pos = A theta
(the C ABI's forward/read/backward replaced by numpy), so the wrapper's
plumbing - theta to seeds, positions out, the vector-Jacobian product back
to theta, the stale-backward check - is checked without a GPU."""
import importlib

import numpy as np
import pytest

torch = pytest.importorskip("torch")


class LinearBackend:
    def __init__(self, A):
        self.A = A  # (n*3, D)
        self.theta = None

    def adjoint_forward(self, world, steps, seeds):
        self.theta = world * steps

    def adjoint_read(self):
        n = self.A.shape[0] // 3
        return (self.A @ self.theta).reshape(n, 3), None, None

    def adjoint_backward(self, grad_pos):
        out = np.zeros(5)
        g = self.A.T @ grad_pos.reshape(-1)
        out[:g.size] = g
        return out


def test_vjp_reaches_theta():
    ag = importlib.import_module("avbd-sandbox_gb300.autograd")
    rng = np.random.default_rng(3)
    A = rng.standard_normal((12, 3))
    be = LinearBackend(A)
    theta = torch.tensor([0.5, -1.0, 2.0], dtype=torch.float64, requires_grad=True)
    seeds = [(0, 0, k, k) for k in range(3)]
    pos = ag.StepFunction.apply(theta, be, lambda th: (th, seeds), 2)
    np.testing.assert_allclose(pos.detach().numpy().reshape(-1), A @ (2 * theta.detach().numpy()))
    w = torch.arange(12, dtype=torch.float64).reshape(4, 3)
    (pos * w).sum().backward()
    np.testing.assert_allclose(theta.grad.numpy(), A.T @ w.numpy().reshape(-1))


def test_rejects_too_many_parameters_and_unused_directions():
    ag = importlib.import_module("avbd-sandbox_gb300.autograd")
    be = LinearBackend(np.zeros((3, 6)))
    with pytest.raises(ValueError):
        ag.StepFunction.apply(torch.zeros(6, dtype=torch.float64), be, lambda th: (th, []), 1)
    with pytest.raises(ValueError):
        ag.StepFunction.apply(torch.zeros(2, dtype=torch.float64), be, lambda th: (th, [(0, 0, 0, 3)]), 1)


def test_stale_backward_raises():
    ag = importlib.import_module("avbd-sandbox_gb300.autograd")
    be = LinearBackend(np.eye(3))
    theta = torch.ones(3, dtype=torch.float64, requires_grad=True)
    first = ag.StepFunction.apply(theta, be, lambda th: (th, []), 1)
    second = ag.StepFunction.apply(theta, be, lambda th: (th, []), 1)
    with pytest.raises(RuntimeError):
        first.sum().backward()
    second.sum().backward()
    np.testing.assert_allclose(theta.grad.numpy(), np.ones(3))
