"""The CPU oracle of the surrogate network: its analytic gradient against
central finite differences (CPU only)."""

import numpy as np

from oracle import mlp as M


def test_oracle_gradient_matches_finite_differences(rng):
    inputs, hidden = 5, 8
    n_params = sum(o * i + o for o, i in M.shapes(inputs, hidden))
    p = rng.normal(scale=0.5, size=n_params)
    xn = rng.normal(size=(6, inputs))
    xo = rng.normal(size=(6, inputs))
    d = rng.normal(size=6)
    loss, g = M.loss_grad(p, xn, xo, d, inputs, hidden)
    eps = 1e-6
    fd = np.empty_like(p)
    for k in range(p.size):
        e = np.zeros_like(p)
        e[k] = eps
        lp, _ = M.loss_grad(p + e, xn, xo, d, inputs, hidden)
        lm, _ = M.loss_grad(p - e, xn, xo, d, inputs, hidden)
        fd[k] = (lp - lm) / (2 * eps)
    np.testing.assert_allclose(g, fd, rtol=1e-5, atol=1e-8)
    assert loss > 0


def test_gelu_matches_its_definition():
    x = np.linspace(-6, 6, 101)
    np.testing.assert_allclose(M.gelu(x), 0.5 * x * (1 + np.tanh(np.sqrt(2 / np.pi)
                                                                  * (x + 0.044715 * x ** 3))))
    h = 1e-6
    np.testing.assert_allclose(M.gelu_grad(x), (M.gelu(x + h) - M.gelu(x - h)) / (2 * h),
                               rtol=1e-6, atol=1e-8)
