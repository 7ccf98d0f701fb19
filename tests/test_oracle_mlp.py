"""The MLP oracle's gradient against central finite differences (float64)."""
import numpy as np

from oracle import mlp_oracle as M


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = rng.normal(0.0, 0.3, M.N_PARAMS)
    x = rng.uniform(0.0, 6.0, (40, M.N_IN))
    t = rng.uniform(5.0, 15.0, 40)
    _, g = M.loss_and_grad(p, x, t)
    n = x.shape[0]
    h = 1e-6
    for i in rng.choice(M.N_PARAMS, 200, replace=False):
        dp = np.zeros(M.N_PARAMS)
        dp[i] = h
        lp, _ = M.loss_and_grad(p + dp, x, t)
        lm, _ = M.loss_and_grad(p - dp, x, t)
        fd = (lp - lm) / (2 * h) / n
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (i, fd, g[i])


def test_oracle_forward_matches_loss():
    rng = np.random.default_rng(4)
    p = rng.normal(0.0, 0.3, M.N_PARAMS)
    x = rng.uniform(0.0, 6.0, (10, M.N_IN))
    t = rng.uniform(5.0, 15.0, 10)
    sse, _ = M.loss_and_grad(p, x, t)
    assert np.isclose(sse, np.sum((M.forward(p, x) - t) ** 2))
