"""Estimator jobs larger than one batch (more than 65535 densities, or more
workspace than the device holds) run as several consecutive engine batches,
each with the views it uses, the workspace given back between them; the
results equal the one-batch results. ENT_MAX_BATCH_INSTANCES lowers the
densities per batch so that small jobs split too. Both contexts of a
comparison take the same pair bodies (1-D range sums, 2-D strip moments for
every instance): 1-D and 2-D results agree to FP64 rounding. 3-D densities
are FP32 sums per tile, and a batch with few tiles splits each tile's
sources into up to 8 shares to fill the GPU, so their summation order
depends on the batch's size: results with 3-D densities (TE, the mixed
entropy batch, transs, dens -D 3) agree to FP32 rounding (1e-7 relative)."""
import numpy as np
import pytest

from entropical_gb300 import Context, workloads
from entropical_gb300.densities import REF_MI, REF_TRANSS

pytestmark = pytest.mark.gpu

BODIES = [6, 7, None]


def _contexts(monkeypatch, per_batch: int):
    one = Context()
    monkeypatch.setenv("ENT_MAX_BATCH_INSTANCES", str(per_batch))
    split = Context()
    monkeypatch.delenv("ENT_MAX_BATCH_INSTANCES")
    for c in (one, split):
        c.set_tuning(pair_variant=BODIES)
    return one, split


def test_mi_te_and_entropy_batches_split(monkeypatch):
    one, split = _contexts(monkeypatch, 5)
    x = workloads.mi_coords(6000, 8, seed=5)
    h = workloads.scott_bandwidth(x, 2)
    mi1, hx1 = one.mi_all_pairs(x, h)
    st1 = one.last_stats()
    mi2, hx2 = split.mi_all_pairs(x, h)
    st2 = split.last_stats()
    assert st1.instances == st2.instances == 8 + 28
    assert st2.kernel_launches > st1.kernel_launches  # 8 runs of at most 5 densities
    assert st2.pair_kernel_ms > 0
    np.testing.assert_allclose(mi2, mi1, rtol=0, atol=1e-12)
    np.testing.assert_allclose(hx2, hx1, rtol=0, atol=1e-12)
    c1, _ = one.mi_all_pairs(x, h, counts=True)
    c2, _ = split.mi_all_pairs(x, h, counts=True)
    assert np.array_equal(c1, c2)  # integer counts: exact

    y, _ = workloads.langevin(n_coords=4, n_steps=4000, seed=3)
    hy = workloads.scott_bandwidth(y, 3)
    te1 = one.te_all_pairs(y, hy, [1, 3])
    te2 = split.te_all_pairs(y, hy, [1, 3])
    assert split.last_stats().instances == 2 * (4 + 4 + 6 + 12)
    np.testing.assert_allclose(te2, te1, rtol=0, atol=1e-6)

    rng = np.random.default_rng(9)
    insts = []
    for q in range(9):
        d = 1 + q % 3
        xi = workloads.mixture_instance(rng, d, int(rng.integers(500, 4000)))
        insts.append((xi, workloads.scott_bandwidth(xi, d)))
    e1 = one.entropy_batch(insts)
    e2 = split.entropy_batch(insts)
    np.testing.assert_allclose(e2, e1, rtol=0, atol=1e-6)


def test_reference_formulas_and_dens_split(monkeypatch):
    one, split = _contexts(monkeypatch, 4)
    x = workloads.mi_coords(3000, 7, seed=6)
    h = workloads.scott_bandwidth(x, 2)
    # transs: the reference's float log of each term moves by an ulp where a
    # 3-D density does
    for est, tau, rel in ((REF_MI, 0, 1e-12), (REF_TRANSS, 2, 1e-5)):
        r1 = one.reference_estimator(x, h, est, tau)
        r2 = split.reference_estimator(x, h, est, tau)
        assert np.max(np.abs(r2 - r1)) <= rel * np.max(np.abs(r1))
    d1 = one.dens_all(x, h, 3)
    d2 = split.dens_all(x, h, 3)
    assert d1.shape == d2.shape == (35, 3000)
    np.testing.assert_allclose(d2, d1, rtol=1e-6, atol=0)


def test_mi_over_more_than_65535_densities():
    """363 coordinates: 363 marginals and 65,703 joints, two batches by the
    instance limit alone. Every MI entry depends only on its two columns, so
    the first 12 columns' block equals the MI of those columns in one batch."""
    x = workloads.mi_coords(300, 363, seed=8)
    h = workloads.scott_bandwidth(x, 2)
    c = Context()
    c.set_tuning(pair_variant=BODIES)
    mi, hx = c.mi_all_pairs(x, h)
    assert c.last_stats().instances == 363 + 363 * 362 // 2
    mi12, hx12 = c.mi_all_pairs(x[:12], h[:12])
    np.testing.assert_allclose(mi[:12, :12], mi12, rtol=0, atol=1e-10)
    np.testing.assert_allclose(hx[:12], hx12, rtol=0, atol=1e-10)
    assert np.all(np.isfinite(mi)) and np.array_equal(mi, mi.T)
