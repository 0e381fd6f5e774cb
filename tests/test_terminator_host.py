"""Learned terminator: the oracle's backpropagation against finite
differences, and the window construction (no GPU)."""
import numpy as np

import oracle.mlp as om
from tdscha_gb300.terminator import windows


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    n_in, n_h, n_out = 6, 9, 4
    n_par = n_in * n_h + n_h + n_h * n_h + n_h + n_h * n_out + n_out
    p = rng.standard_normal(n_par) * 0.3
    x = rng.standard_normal((7, n_in))
    t = rng.standard_normal((7, n_out))
    loss, g = om.loss_grad(p, x, t, n_in, n_h, n_out)
    fd = np.zeros_like(p)
    for i in range(n_par):
        e = np.zeros_like(p)
        e[i] = 1e-6
        fd[i] = (om.loss_grad(p + e, x, t, n_in, n_h, n_out)[0]
                 - om.loss_grad(p - e, x, t, n_in, n_h, n_out)[0]) / 2e-6
    np.testing.assert_allclose(g, fd, rtol=1e-6, atol=1e-9)


def test_windows():
    a = np.arange(100.0)
    b = 1000 + np.arange(100.0)
    x, t = windows(a, b, 2.0, k_min=32, window=32, horizon=64)
    assert x.shape == (5, 66) and t.shape == (5, 128)
    ma, mb = np.mean(a[0:32] / 2), np.mean(b[0:32] / 2)
    np.testing.assert_allclose(x[0, :32], a[0:32] / 2 - ma)
    np.testing.assert_allclose(x[0, 32:64], b[0:32] / 2 - mb)
    np.testing.assert_allclose(x[0, 64:], [ma, mb])
    ma4 = np.mean(a[4:36] / 2)
    np.testing.assert_allclose(t[4, :64], a[36:100] / 2 - ma4)
