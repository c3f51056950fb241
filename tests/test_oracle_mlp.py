"""The FP64 MLP oracle itself: analytic gradients against finite differences."""
import numpy as np

from oracle import mlp_ref as R


def test_oracle_gradient_finite_differences():
    rng = np.random.default_rng(0)
    n_params = sum(int(np.prod(s)) for _, s in R.SHAPES)
    assert n_params == 21123
    p = (rng.standard_normal(n_params) * 0.1).astype(np.float32)
    # keep the check inside one BF16 rounding cell: perturb only biases
    mu, sd = np.zeros(32, np.float32), np.ones(32, np.float32)
    X = rng.standard_normal((16, 32)).astype(np.float32)
    T = rng.standard_normal((16, 3)).astype(np.float32)
    M = (rng.random((16, 3)) < 0.7).astype(np.float32)
    loss, g = R.loss_and_grad(p, mu, sd, X, T, M)
    off_b3 = n_params - 3
    off_b2 = 128 * 32 + 128 + 128 * 128
    for i in [off_b3, off_b3 + 2, off_b2 + 5, 128 * 32 + 7]:
        e = np.zeros(n_params, np.float64)
        e[i] = 1e-3
        lp, _ = R.loss_and_grad(p.astype(np.float64) + e, mu, sd, X, T, M)
        lm, _ = R.loss_and_grad(p.astype(np.float64) - e, mu, sd, X, T, M)
        assert abs((lp - lm) / 2e-3 - g[i]) < 1e-6 * max(1, abs(g[i])) + 1e-7
