"""The FP64 MLP oracle itself: analytic gradients against finite differences;
and the committed network weights run through it on the CPU."""
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


def test_shipped_network_predicts_the_searchs_constant_ratio():
    """The committed weights (entropical_gb300/data/bandwidth_mlp.npz) have the
    library's layout, and the FP64 oracle forward pass on oracle features of
    fresh mixtures predicts log(h / h0) = log(2 - 1.9/512) for every used
    dimension: the reference's AMISE search always returns that ratio, since
    its objective falls monotonically in h, so that is what the network learned."""
    from entropical_gb300 import _native, learned, workloads
    z = np.load(learned.DEFAULT_WEIGHTS)
    assert z["params"].shape == (int(_native.load().ent_mlp_param_count()),) == (21123,)
    assert z["mu"].shape == z["sd"].shape == (32,)
    assert np.all(np.isfinite(z["params"])) and np.all(z["sd"] > 0)
    rng = np.random.default_rng(3)
    target = np.log(learned.CONSTANT_RATIO)
    for q in range(9):
        d = 1 + q % 3
        x = workloads.mixture_instance(rng, d, 3000)
        y = R.forward(z["params"], z["mu"], z["sd"], R.features(x)[None].astype(np.float32))[3][0]
        assert np.all(np.abs(y[:d] - target) < 1e-4), (d, y)
