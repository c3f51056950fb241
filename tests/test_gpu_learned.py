"""The learned warm start: feature kernel, MLP forward/backward against the
FP64 oracle, device training, and what the trained network gains over the
search without it."""
import numpy as np
import pytest

from entropical_gb300 import learned, workloads
from entropical_gb300.densities import HEST_AMISE
from oracle import mlp_ref as R
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_features_match_oracle(ctx):
    rng = np.random.default_rng(5)
    items = [workloads.mixture_instance(rng, d, n) for d, n in [(1, 3000), (2, 5000), (3, 4000)]]
    F = learned.features(ctx, items)
    for f, x in zip(F, items):
        ref = R.features(x)
        assert np.allclose(f, ref, rtol=2e-4, atol=2e-5), np.abs(f - ref).max()


def test_forward_and_gradients_match_oracle(ctx):
    rng = np.random.default_rng(6)
    net = learned.BandwidthMLP(ctx, seed=3)
    p, _, _ = net.get_params()
    mu = rng.standard_normal(32).astype(np.float32)
    sd = rng.uniform(0.5, 2, 32).astype(np.float32)
    p = p + (rng.standard_normal(p.size) * 0.01).astype(np.float32)
    net.set_params(p, mu, sd)
    X = rng.standard_normal((300, 32)).astype(np.float32) * sd + mu
    T = rng.standard_normal((300, 3)).astype(np.float32)
    M = (rng.random((300, 3)) < 0.8).astype(np.float32)
    y = net.forward(X)
    *_, yr, _ = R.forward(p, mu, sd, X)
    assert np.allclose(y, yr, rtol=1e-4, atol=1e-5)
    g, loss = net.gradients(X, T, M)
    lr, gr = R.loss_and_grad(p, mu, sd, X, T, M)
    assert abs(loss - lr) / lr < 1e-5
    assert np.linalg.norm(g - gr) / np.linalg.norm(gr) < 1e-4


def test_training_and_warm_start_gain(ctx):
    # small training set of generated mixtures labelled by the full search
    X, T, M = learned.make_dataset(ctx, 240, seed=11, n_min=2000, n_max=20000, chunk=120)
    net, losses = learned.train(ctx, X, T, M, epochs=40, batch=64, lr=3e-3)
    assert losses[-1] < 0.05 * losses[0]
    rng = np.random.default_rng(99)
    held = [workloads.mixture_instance(rng, int(rng.integers(1, 4)), int(rng.integers(3000, 30000)))
            for _ in range(24)]
    h_full, st_full = learned.hestimate_full(ctx, held)
    h_warm, st_warm = learned.hestimate_learned(ctx, net, held, skip_levels=6)
    assert np.array_equal(h_full, h_warm)
    evals_full = sum(s["conv_evals"] for row in st_full for s in row)
    evals_warm = sum(s["conv_evals"] for row in st_warm for s in row)
    # 16 convolutions per column without the network, 4 with it
    assert evals_warm * 4 == evals_full
    # The constant-offset warm start (no network) does exactly as well: the
    # reference's AMISE objective falls monotonically in h, so every label is
    # the same ratio and the network has nothing else to learn.
    h_const, st_const = learned.hestimate_constant(ctx, held, skip_levels=6)
    assert np.array_equal(h_full, h_const)
    evals_const = sum(s["conv_evals"] for row in st_const for s in row)
    assert evals_const == evals_warm
    assert np.allclose(T[M > 0], np.log(learned.CONSTANT_RATIO), atol=1e-6)
    # the bandwidth search agrees with the restated reference search
    x0 = held[0][0]
    assert O.hestimate_amise(x0)[0] == h_full[0, 0]


def test_held_out_evaluation_against_fp64(ctx):
    """The committed network on held-out mixtures: the three arms (full
    search, network, constant offset) give the same bandwidths, the warm
    starts never fall back, and the entropies at those bandwidths agree with
    the FP64 oracle's entropy at the full search's bandwidths."""
    net = learned.BandwidthMLP.load(ctx)
    held = learned.generate(24, seed=4242, n_min=3000, n_max=20000)
    ev = learned.evaluate(ctx, net, held)
    cols = ev["columns"]
    assert ev["none"]["conv_evals"] == 16 * cols
    for arm in ("network", "constant"):
        assert ev[arm]["identical_h"] and ev[arm]["fallbacks"] == 0
        assert ev[arm]["conv_evals"] == 4 * cols
        assert ev[arm]["max_abs_dH_vs_full"] == 0.0
    for q, x in enumerate(held):
        d = x.shape[0]
        ref = O.entropy_fp64(x, ev["h_full"][q, :d])
        assert abs(ev["H_full"][q] - ref) < 1e-6, (q, ev["H_full"][q], ref)
