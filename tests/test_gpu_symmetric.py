"""GPU parity of the symmetric pair bodies (pair_variant 4 and 5: every
unordered pair evaluated once and added to both points) against the FP64
oracle, the reference's golden outputs and the ordered bodies.

Tolerances as for the ordered path: densities 1e-5 relative per point,
entropies / MI / TE 1e-6 nats absolute against FP64; symmetric vs ordered
batches 2e-6 nats (each is within 1e-6 of FP64; they differ by summation
order only); support counts exact (counting uses the ordered body)."""
import numpy as np
import pytest

from entropical_gb300 import workloads
from oracle import oracle as O

pytestmark = pytest.mark.gpu

REL = 1e-5
SYM = (4, 5)


def rel_err(a, b):
    return np.max(np.abs(np.asarray(a) - np.asarray(b)) / np.abs(np.asarray(b)))


@pytest.fixture(params=SYM)
def sym_ctx(request):
    from entropical_gb300 import Context
    c = Context(0)
    c.set_tuning(pair_variant=request.param)
    assert c.tuning()["pair_variant_by_dim"] == [request.param] * 3
    yield c
    c.close()


@pytest.mark.parametrize("d", [1, 2, 3])
@pytest.mark.parametrize("n", [1, 2, 63, 64, 65, 1000, 20000])
def test_sym_fp64_shapes(sym_ctx, d, n):
    rng = np.random.default_rng(3000 * d + n)
    x = rng.standard_normal((3, n)).astype(np.float32)
    h = rng.uniform(0.15, 0.6, d).astype(np.float32)
    cols = list(rng.permutation(3)[:d])
    p = sym_ctx.combined_densities(x, None, cols, h)
    assert rel_err(p, O.density_fp64(O.repack(x, cols), h)) < REL


@pytest.mark.parametrize("d", [1, 2, 3])
def test_sym_ties_and_extreme_bandwidths(sym_ctx, d):
    rng = np.random.default_rng(90 + d)
    # heavy ties: a third of the points on one value per column, quantised rest
    x = np.round(rng.standard_normal((3, 5000)) * 8) / 8
    x[:, ::3] = 0.5
    x = x.astype(np.float32)
    cols = [0, 1, 2][:d]
    for hv in (0.125, 1e-6, 50.0):
        p = sym_ctx.combined_densities(x, None, cols, [hv] * d)
        assert rel_err(p, O.density_fp64(O.repack(x, cols), [hv] * d)) < REL
    # all points equal: every pair in support, one strip, one window
    z = np.full((3, 700), -1.25, np.float32)
    p = sym_ctx.combined_densities(z, None, cols, [0.3] * d)
    assert rel_err(p, O.density_fp64(O.repack(z, cols), [0.3] * d)) < REL


@pytest.mark.parametrize("case", ["d1", "d2", "d3", "lag"])
def test_sym_golden_reference(sym_ctx, golden, case):
    g = golden
    if case == "d1":
        p = sym_ctx.combined_densities(g["d1_x"], None, [0], g["d1_h"])
        ref = g["d1_p"]
    elif case == "d2":
        p = sym_ctx.combined_densities(g["d2_x"], None, [0, 1], g["d2_h"])
        ref = g["d2_p"]
    elif case == "d3":
        p = sym_ctx.combined_densities(g["d2_x"], None, [0, 1, 2], g["d3_h"])
        ref = g["d3_p"]
    else:
        p = sym_ctx.combined_densities(g["d2_x"], None, list(g["lag_cols"]), g["lag_h"],
                                       list(g["lag_tau"]))
        ref = g["lag_p"]
    assert rel_err(p, ref) < REL


def test_sym_mi_batch(sym_ctx, ctx):
    x = workloads.mi_coords(8000, 6, seed=12)
    h = workloads.scott_bandwidth(x, 2)
    mi, hx = sym_ctx.mi_all_pairs(x, h)
    mi0, hx0 = ctx.mi_all_pairs(x, h)
    assert np.max(np.abs(mi - mi0)) < 2e-6 and np.max(np.abs(hx - hx0)) < 2e-6
    for i in range(6):
        assert abs(hx[i] - O.entropy_fp64(x[i:i + 1], [h[i]])) < 1e-6
    for i, j in [(0, 3), (4, 5), (1, 2)]:
        assert abs(mi[i, j] - O.mi_fp64(x[i], x[j], h[i], h[j])) < 1e-6
    assert np.all(mi == mi.T) and np.all(np.diag(mi) == 0)


def test_sym_uneven_batch(sym_ctx, ctx):
    rng = np.random.default_rng(21)
    insts = []
    for _ in range(20):
        d = int(rng.integers(1, 4))
        n = int(np.exp(rng.uniform(np.log(40), np.log(25000))))
        x = workloads.mixture_instance(rng, d, n)
        insts.append((x, workloads.scott_bandwidth(x, d)))
    H = sym_ctx.entropy_batch(insts)
    H0 = ctx.entropy_batch(insts)
    assert np.max(np.abs(H - H0)) < 2e-6
    for q in (0, 7, 13):
        x, h = insts[q]
        assert abs(H[q] - O.entropy_fp64(x, h)) < 1e-6


def test_sym_te_batch(sym_ctx, ctx):
    x, _ = workloads.langevin(n_coords=4, n_steps=5000, seed=5)
    h = workloads.scott_bandwidth(x, 3)
    te = sym_ctx.te_all_pairs(x, h, [1, 4])
    te0 = ctx.te_all_pairs(x, h, [1, 4])
    assert np.max(np.abs(te - te0)) < 2e-6
    assert abs(te[1, 2, 0] - O.te_fp64(x[0], x[2], 4, h[0], h[2])) < 1e-6


@pytest.mark.parametrize("d", [1, 2, 3])
def test_sym_support_counts_exact(sym_ctx, ctx, d):
    rng = np.random.default_rng(5 + d)
    x = rng.standard_normal((3, 3000)).astype(np.float32)
    cols = [1, 2, 0][:d]
    h = [0.3, 0.35, 0.4][:d]
    c = sym_ctx.support_counts(x, None, cols, h)
    assert np.array_equal(c, ctx.support_counts(x, None, cols, h))
    cnt, c1 = sym_ctx.mi_all_pairs(x, [0.3, 0.3, 0.3], counts=True)
    assert c1[0] == sym_ctx.support_counts(x, None, [0], [0.3]).sum()


@pytest.mark.parametrize("cells3", [1, 2])
def test_sym_3d_cell_sizes(cells3):
    """Strips of 1 or 2 cells per bandwidth in dimensions 1 and 2 (5 x 5
    neighbour strips, 25 source runs per tile at 2) give the same densities."""
    from entropical_gb300 import Context
    rng = np.random.default_rng(70 + cells3)
    x = rng.standard_normal((3, 9000)).astype(np.float32)
    with Context(0) as c:
        c.set_tuning(cells_per_h3=cells3)
        assert c.tuning()["cells_per_h3"] == cells3
        for v in (2, 4):
            c.set_tuning(pair_variant=v)
            p = c.combined_densities(x, None, [0, 1, 2], [0.2, 0.3, 0.25])
            assert rel_err(p, O.density_fp64(O.repack(x, [0, 1, 2]), [0.2, 0.3, 0.25])) < REL
        cnt = c.support_counts(x, None, [0, 1, 2], [0.2, 0.3, 0.25])
    with Context(0) as c1:
        c1.set_tuning(cells_per_h3=1)
        assert np.array_equal(cnt, c1.support_counts(x, None, [0, 1, 2], [0.2, 0.3, 0.25]))
