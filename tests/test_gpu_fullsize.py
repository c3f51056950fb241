"""The benchmark configurations at their full sizes, checked through
properties that do not need an O(n^2) oracle: densities at sampled targets
against the FP64 oracle (1e-5 relative), the batch against per-instance
plain calls (1e-7 nats: the same terms, other FP32 partial sums), entropies
of the smallest instances against FP64 (1e-6 nats), support counts against
the FP64 count (exact)."""
import numpy as np
import pytest

from entropical_gb300 import workloads
from oracle import oracle as O

pytestmark = pytest.mark.gpu

REL = 1e-5


def rel_err(a, b):
    return np.max(np.abs(np.asarray(a) - np.asarray(b)) / np.abs(np.asarray(b)))


def test_te_config_full_size(ctx):
    """Transfer entropy, 32 coords x 200k Langevin frames, lags {1, 5, 10}."""
    x, _ = workloads.langevin(32, 200_000, seed=11)
    h = workloads.scott_bandwidth(x, 3)
    taus = [1, 5, 10]
    te = ctx.te_all_pairs(x, h, taus)
    assert te.shape == (3, 32, 32) and np.all(np.isfinite(te))
    assert np.all(np.diag(te[0]) == 0)
    rng = np.random.default_rng(7)
    for q, (i, j) in enumerate([(0, 5), (17, 3), (30, 29)]):
        tau = taus[q]
        n = 200_000 - tau
        # the 3-D density (y+, y, x) at sampled targets against FP64
        p3 = ctx.combined_densities(x, None, [i, i, j], [h[i], h[i], h[j]], [tau, 0, 0])
        t = rng.choice(n, 2000, replace=False)
        sel = np.stack([x[i][tau:tau + n], x[i][:n], x[j][:n]])
        f = O.density_fp64(sel, [h[i], h[i], h[j]], targets=t)
        assert rel_err(p3[t], f) < REL
        # the batch against the plain path's four entropies
        xn = np.ascontiguousarray(x[:, :n])
        H1 = -np.mean(np.log(ctx.combined_densities(xn, None, [i], [h[i]])))
        H2 = -np.mean(np.log(ctx.combined_densities(xn, None, [i, j], [h[i], h[j]])))
        Hl = -np.mean(np.log(ctx.combined_densities(x, None, [i, i], [h[i], h[i]], [tau, 0])))
        H3 = -np.mean(np.log(p3))
        assert abs(te[q, i, j] - (H2 + Hl - H3 - H1)) < 1e-7


def test_uneven_config_full_size(ctx):
    """512 instances, d in {1,2,3}, n log-uniform in [2k, 500k]."""
    ub = workloads.uneven_batch(512, seed=5)
    H = ctx.entropy_batch(ub)
    assert H.shape == (512,) and np.all(np.isfinite(H))
    order = np.argsort([x.shape[1] for x, _ in ub])
    for q in order[:6]:  # the smallest instances: FP64 entropy
        x, h = ub[q]
        assert abs(H[q] - O.entropy_fp64(x, h)) < 1e-6
    rng = np.random.default_rng(3)
    for q in rng.choice(512, 12, replace=False):  # batch == plain calls
        x, h = ub[q]
        p = ctx.combined_densities(x, None, list(range(x.shape[0])), h)
        assert abs(H[q] + np.mean(np.log(p))) < 1e-7
    # support counts of a mid-size instance: exact against the FP64 count
    q = order[40]
    x, h = ub[q]
    c = ctx.entropy_batch([(x, h)], counts=True)[0]
    assert c == O.support_count_fp64(x, h)


def test_mi_config_full_size_batch_vs_plain(ctx):
    """All-pairs MI 64 x 100k: the batch equals the plain path on sampled pairs."""
    x = workloads.mi_coords(100_000, 64, seed=2024)
    h = workloads.scott_bandwidth(x, 2)
    mi, hx = ctx.mi_all_pairs(x, h)
    assert np.all(np.isfinite(mi)) and np.all(mi == mi.T)
    for i, j in [(0, 1), (13, 52), (40, 63)]:
        pij = ctx.combined_densities(x, None, [i, j], [h[i], h[j]])
        assert abs(mi[i, j] - (hx[i] + hx[j] + np.mean(np.log(pij)))) < 1e-7
    assert abs(mi[0, 1] - O.mi_fp64(x[0], x[1], h[0], h[1])) < 1e-6
