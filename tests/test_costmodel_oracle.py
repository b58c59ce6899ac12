"""CPU: the cost model's oracle gradient (oracle/mlp.py) against central
finite differences, and the candidate / feature entry points' host logic."""
import numpy as np
import pytest

from oracle import mlp as omlp

F = 48


@pytest.mark.parametrize("h,n", [(8, 5), (16, 40), (64, 12)])
def test_oracle_gradient_finite_differences(h, n):
    rng = np.random.default_rng(h * 100 + n)
    p = rng.standard_normal(h * F + h + h * h + h + h + 1) * 0.3
    X = rng.standard_normal((n, F))
    y = rng.standard_normal(n)
    loss, g = omlp.loss_grad(p, X, y, F, h)
    assert np.isclose(loss, 0.5 * np.mean((omlp.forward(p, X, F, h) - y) ** 2))
    idx = rng.choice(p.size, 60, replace=False)
    eps = 1e-6
    for i in idx:
        d = np.zeros_like(p)
        d[i] = eps
        num = (omlp.loss_grad(p + d, X, y, F, h)[0] - omlp.loss_grad(p - d, X, y, F, h)[0]) / (2 * eps)
        assert abs(num - g[i]) <= 1e-6 + 1e-5 * abs(g[i]), (i, num, g[i])


def test_oracle_layout_roundtrip():
    h = 4
    p = np.arange(h * F + h + h * h + h + h + 1, dtype=np.float64)
    W1, b1, W2, b2, W3, b3 = omlp.unpack(p, F, h)
    assert W1.shape == (h, F) and W2.shape == (h, h) and W3.shape == (h,)
    assert W1[0, 0] == 0 and b1[0] == h * F and b3 == p[-1]
