"""GPU parity of the 2-D strip-moment body (pair_variant_by_dim[1] = 7):
strips wholly inside a target's y-support are summed from exact fixed-point
moment prefix sums, the strips crossing its edge pair by pair.

Checked against the FP64 oracle at 1e-5 relative per point, against the
symmetric pair body at 1e-6 relative, and through the MI / TE / entropy
batches at 1e-6 nats against FP64, on data chosen to break moments taken in
floating point: large offsets, heavy ties, outliers, spreads far below the
bandwidth, self-only supports and very unequal bandwidths."""
import numpy as np
import pytest

from entropical_gb300 import workloads
from oracle import oracle as O

pytestmark = pytest.mark.gpu

REL = 1e-5
MOM = [None, 7, None]


@pytest.fixture
def mctx():
    from entropical_gb300 import Context
    c = Context(0)
    c.set_tuning(pair_variant=MOM)
    assert c.tuning()["pair_variant_by_dim"][1] == 7
    yield c
    c.close()


def rel_err(a, b):
    return np.max(np.abs(np.asarray(a) - np.asarray(b)) / np.abs(np.asarray(b)))


def _cases():
    rng = np.random.default_rng(91)
    base = rng.standard_normal((2, 20000)).astype(np.float32)
    return {
        "normal": (base, (0.2, 0.3)),
        "offset": (base + np.float32([[1000.0], [-2.5e4]]), (0.15, 0.2)),
        "ties": (np.round(base, 1).astype(np.float32), (0.12, 0.3)),
        "outliers": (np.concatenate([base[:, :6000], np.float32([[1e30, -4e22, 3.0],
                                                                 [2.0, 5e25, -1e28]])], axis=1),
                     (0.25, 0.25)),
        "narrow": (rng.normal(3.0, 1e-4, (2, 3000)).astype(np.float32), (0.5, 0.5)),
        "self_only": (np.stack([np.arange(400, dtype=np.float32),
                                np.arange(400, dtype=np.float32)[::-1]]), (0.4, 0.4)),
        "unequal_h": (base[:, :8000], (0.02, 2.5)),
        "tiny_n": (np.float32([[0.1, 0.3], [0.2, -0.1]]), (0.5, 0.5)),
        "one": (np.float32([[1.0], [2.0]]), (0.3, 0.3)),
    }


@pytest.mark.parametrize("name", list(_cases()))
def test_moments_fp64(mctx, name):
    x, h = _cases()[name]
    p = mctx.combined_densities(x, None, [0, 1], list(h))
    ref = O.density_fp64(x, list(h))
    assert rel_err(p, ref) < REL


@pytest.mark.parametrize("n", [2, 63, 64, 65, 129, 5000])
def test_moments_shapes(mctx, n):
    rng = np.random.default_rng(700 + n)
    x = rng.standard_normal((2, n)).astype(np.float32)
    h = rng.uniform(0.15, 0.6, 2).astype(np.float32)
    assert rel_err(mctx.combined_densities(x, None, [0, 1], h), O.density_fp64(x, h)) < REL


@pytest.mark.parametrize("name", ["normal", "offset", "ties", "unequal_h"])
def test_moments_vs_symmetric_pair_body(mctx, ctx, name):
    x, h = _cases()[name]
    a = mctx.combined_densities(x, None, [0, 1], list(h))
    b = ctx.combined_densities(x, None, [0, 1], list(h))
    assert rel_err(a, b) < 1e-6


def test_moments_mi_batch(mctx):
    x = workloads.mi_coords(20000, 8, seed=44)
    h = workloads.scott_bandwidth(x, 2)
    mi, hx = mctx.mi_all_pairs(x, h)
    for i, j in [(0, 1), (2, 7), (5, 6)]:
        assert abs(mi[i, j] - O.mi_fp64(x[i], x[j], h[i], h[j])) < 1e-6


def test_moments_te_and_entropy_batch(mctx):
    x, _ = workloads.langevin(4, 6000, seed=3)
    h = workloads.scott_bandwidth(x, 3)
    te = mctx.te_all_pairs(x, h, [2])
    i, j, tau = 1, 3, 2
    n = 6000 - tau
    H = lambda sel, hh: O.entropy_fp64(np.ascontiguousarray(sel), hh)  # noqa: E731
    ref = (H(np.stack([x[i][:n], x[j][:n]]), [h[i], h[j]])
           + H(np.stack([x[i][tau:tau + n], x[i][:n]]), [h[i], h[i]])
           - H(np.stack([x[i][tau:tau + n], x[i][:n], x[j][:n]]), [h[i], h[i], h[j]])
           - H(x[i][None, :n], [h[i]]))
    assert abs(te[0, i, j] - ref) < 1e-6
    rng = np.random.default_rng(17)
    items = [(workloads.mixture_instance(rng, 2, n), None) for n in (300, 4000, 20000)]
    items = [(xx, workloads.scott_bandwidth(xx, 2)) for xx, _ in items]
    Hb = mctx.entropy_batch(items)
    for q, (xx, hh) in enumerate(items):
        assert abs(Hb[q] - O.entropy_fp64(xx, hh)) < 1e-6


def test_moments_counts_use_pair_body(mctx):
    # generic data: ties at exactly the bandwidth distance would make the
    # FP64 count and the kernels' float support test disagree on the edge
    x, h = _cases()["normal"]
    c = mctx.entropy_batch([(x[:, :5000], np.float32(h))], counts=True)[0]
    assert c == O.support_count_fp64(x[:, :5000], h)


def test_moment_variant_only_for_two_dimensions(ctx):
    from entropical_gb300._native import NativeError
    with pytest.raises(NativeError):
        ctx.set_tuning(pair_variant=[7, None, None])
    with pytest.raises(NativeError):
        ctx.set_tuning(pair_variant=[None, None, 7])
    with pytest.raises(NativeError):
        ctx.set_tuning(pair_variant=[None, 6, None])


@pytest.mark.parametrize("name,kind,tau", [("mi", 1, 0), ("transs", 2, 3), ("kldiv", 5, 0)])
def test_moments_reference_estimators(mctx, name, kind, tau):
    """The reference's estimator formulas (per-point output epilogue of the
    moment kernel) against the FP64 oracle, as for the pair bodies."""
    x = workloads.mi_coords(4000, 5, seed=31)
    h = workloads.scott_bandwidth(x, 2)
    r = mctx.reference_estimator(x, h, kind, tau)
    f, bnd = O.reference_estimator_fp64(x, h, name, tau, bound=True)
    assert np.all(np.abs(r - f) <= 1e-6 * bnd + 1e-12)


def test_moments_dens_all_2d(mctx):
    """dens -D 2 (per-point output and the plain-sum epilogue) against FP64."""
    x = workloads.mi_coords(3000, 4, seed=5)
    h = workloads.scott_bandwidth(x, 2)
    d2 = mctx.dens_all(x, h, 2)
    pairs = [(i, j) for i in range(4) for j in range(i + 1, 4)]
    assert d2.shape == (len(pairs), 3000)
    for r, (i, j) in enumerate(pairs):
        p = O.density_fp64(np.stack([x[i], x[j]]), [h[i], h[j]])
        assert np.max(np.abs(d2[r] - p / p.sum()) / (p / p.sum())) < 1e-5
    assert np.allclose(d2.sum(1), 1.0, rtol=1e-12)


def test_moments_default_rule(ctx):
    """Without an explicit choice, a call below 2 M 2-D points runs the
    symmetric pair body and a larger batch the strip moments; both agree."""
    x = workloads.mi_coords(40000, 12, seed=9)
    h = workloads.scott_bandwidth(x, 2)
    assert ctx.tuning()["pair_variant_by_dim"][1] == 7
    small, _ = ctx.mi_all_pairs(x[:3], h[:3])       # 3 x 40k 2-D points
    k_small = ctx.last_stats().kernel_launches
    big, _ = ctx.mi_all_pairs(x, h)                 # 66 x 40k = 2.64 M 2-D points
    k_big = ctx.last_stats().kernel_launches
    assert k_big > k_small                           # the moment kernels launched
    assert np.allclose(big[:3, :3], small, rtol=0, atol=2e-6)
    for i, j in [(0, 1), (4, 11)]:
        assert abs(big[i, j] - O.mi_fp64(x[i], x[j], h[i], h[j])) < 1e-6


def test_moments_mixed_batch_per_instance_choice(ctx):
    """A default batch above 2 M 2-D points with instances of very different
    support per target: the device picks the body per instance (moments for
    wide supports, the symmetric pair kernel for narrow ones); entropies
    match a symmetric-only context (itself checked against FP64 above)."""
    from entropical_gb300 import Context
    rng = np.random.default_rng(23)
    items = []
    for q in range(24):
        n = 120_000
        x = rng.standard_normal((2, n)).astype(np.float32)
        if q % 2:
            x = np.tanh(2.5 * x).astype(np.float32)   # concentrated: wide support
            h = np.float32([0.3, 0.3])
        else:
            h = np.float32([0.02, 0.03])               # narrow support
        items.append((x, h))
    H = ctx.entropy_batch(items)
    with Context(0) as s:
        s.set_tuning(pair_variant=[None, 4, None])
        Hs = s.entropy_batch(items)
    assert np.max(np.abs(H - Hs)) < 2e-6
