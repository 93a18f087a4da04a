"""The host restatement of the control-variate network (oracle/mlp_oracle.py)
pinned by first principles: its gradient equals central finite differences
of its loss, and gelu' of gelu."""
import numpy as np

from oracle import mlp_oracle as O


def test_gelu_derivative():
    z = np.linspace(-6, 6, 101)
    h = 1e-6
    fd = (O.gelu(z + h) - O.gelu(z - h)) / (2 * h)
    np.testing.assert_allclose(O.gelu_d(z), fd, rtol=1e-7, atol=1e-9)


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    F, H, B = 5, 7, 11
    P = H * F + H + H * H + H + H + 1
    p = rng.normal(size=P) * 0.5
    x = rng.normal(size=(B, F))
    t = rng.normal(size=B)
    loss, g = O.loss_and_grad(p, x, t, H)
    fd = np.empty(P)
    for k in range(P):
        e = np.zeros(P)
        e[k] = 1e-6
        fd[k] = (O.loss_and_grad(p + e, x, t, H)[0] - O.loss_and_grad(p - e, x, t, H)[0]) / 2e-6
    np.testing.assert_allclose(g, fd, rtol=1e-6, atol=1e-9)


def test_adam_first_step_is_signed_lr():
    p, g = np.array([1.0, -2.0, 3.0]), np.array([0.5, -1e-3, 2.0])
    p1, m, v = O.adam(p, g, np.zeros(3), np.zeros(3), 1e-2, 1)
    np.testing.assert_allclose(p1, p - 1e-2 * np.sign(g), rtol=1e-6)
