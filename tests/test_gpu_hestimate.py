"""GPU parity of the AMISE convolution and the on-device bandwidth search
against the reference (golden fixtures) and the FP64 oracle."""
import numpy as np
import pytest

from entropical_gb300 import workloads
from entropical_gb300.densities import HEST_AMISE, HEST_AMISE_WARM, HEST_THUMB
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_convolution_golden(ctx, golden):
    for h, v in zip(golden["conv_h"], golden["conv_v"]):
        c = ctx.epa_convolution(golden["conv_x"], float(h))
        assert abs(c - v) / v < 2e-6


@pytest.mark.parametrize("n", [1, 7, 5000, 60000])
def test_convolution_fp64(ctx, n):
    x = np.sort(workloads.gmm_1d(n, seed=n))
    for h in (0.01, 0.2, 3.0):
        assert abs(ctx.epa_convolution(x, h) - O.epa_conv_fp64(x, h)) / O.epa_conv_fp64(x, h) < 2e-6


def test_convolution_offset_ties_and_size(ctx):
    """Range sums from centred FP64 prefix sums: a column far from zero, a
    column of heavy ties and a longer column, each against the FP64 oracle."""
    base = workloads.gmm_1d(20000, seed=31)
    cases = [(np.sort(base + np.float32(1000.0)), (0.02, 0.5)),
             (np.sort(np.round(base, 2).astype(np.float32)), (0.004, 0.05, 0.6)),
             (np.sort(workloads.gmm_1d(200000, seed=32)), (0.005, 0.08))]
    for x, hs in cases:
        for h in hs:
            ref = O.epa_conv_fp64(x, h)
            assert abs(ctx.epa_convolution(x, h) - ref) / ref < 2e-6


def test_convolution_unsorted_input(ctx):
    x = workloads.gmm_1d(3000, seed=4)
    assert abs(ctx.epa_convolution(x, 0.1) - O.epa_conv_fp64(np.sort(x), 0.1)) < 1e-6


def test_hestimate_golden(ctx, golden):
    h, st = ctx.hestimate(golden["hest_x"], HEST_AMISE)
    assert np.array_equal(h, golden["hest_amise"])
    assert all(s["conv_evals"] == 16 for s in st)
    t, _ = ctx.hestimate(golden["hest_x"], HEST_THUMB)
    assert np.array_equal(t, golden["hest_thumb"])


def test_hestimate_matches_restatement(ctx):
    rng = np.random.default_rng(12)
    cols = np.stack([workloads.mixture_instance(rng, 1, 5000)[0] for _ in range(6)])
    h, _ = ctx.hestimate(cols, HEST_AMISE)
    for c, hc in zip(cols, h):
        assert O.hestimate_amise(c, exact=False)[0] == hc
        assert O.thumb_ref(c) * (2 - 1.9 / 512) == pytest.approx(hc, rel=1e-6)


def test_warm_start_saves_levels_and_is_exact(ctx):
    rng = np.random.default_rng(13)
    cols = np.stack([workloads.mixture_instance(rng, 1, 20000)[0] for _ in range(5)])
    full, sf = ctx.hestimate(cols, HEST_AMISE)
    h0 = np.array([s["h0"] for s in sf], np.float32)
    warm, sw = ctx.hestimate(cols, HEST_AMISE_WARM, h_init=1.99 * h0, skip_levels=6)
    assert np.array_equal(warm, full)
    assert all(s["conv_evals"] == 4 and s["warm_converged"] == 1 for s in sw)
    # a poor start ends against an inner node edge and falls back
    bad, sb = ctx.hestimate(cols, HEST_AMISE_WARM, h_init=0.3 * h0, skip_levels=6)
    assert np.array_equal(bad, full)
    assert all(s["warm_converged"] == 0 and s["conv_evals"] == 20 for s in sb)


def test_hestimate_device_column_subset(ctx):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(21)
    cols = np.stack([workloads.mixture_instance(rng, 1, 7000)[0] for _ in range(5)])
    full, _ = ctx.hestimate(cols, HEST_AMISE)
    d = torch.from_numpy(cols).cuda()
    sel = np.array([4, 1, 3], np.uint32)
    h = np.zeros(3, np.float32)
    import ctypes as C
    from entropical_gb300._native import HestStats, c_f32_p, c_u32_p
    st = (HestStats * 3)()
    ctx.check(ctx.lib.ent_hestimate_device(ctx.handle, C.c_void_p(d.data_ptr()), 7000, 5,
                                           sel.ctypes.data_as(c_u32_p), 3, HEST_AMISE, None, 0,
                                           h.ctypes.data_as(c_f32_p), C.cast(st, C.c_void_p)))
    assert np.array_equal(h, full[sel])


def test_hestimate_instance_batch(ctx):
    from entropical_gb300 import learned
    rng = np.random.default_rng(22)
    items = [workloads.mixture_instance(rng, d, n) for d, n in [(2, 4000), (1, 9000), (3, 3000)]]
    h, st = learned.hestimate_full(ctx, items)
    for q, x in enumerate(items):
        ref, _ = ctx.hestimate(x, HEST_AMISE)
        assert np.array_equal(h[q, :x.shape[0]], ref)
        assert np.all(h[q, x.shape[0]:] == 0)


def test_hestimate_over_more_than_65535_columns(ctx):
    """70,000 columns run as two passes (the per-column kernels index columns
    by the grid's y dimension). Each column's search depends on that column
    alone, so the bandwidths equal a search over a few of them, bit for bit."""
    rng = np.random.default_rng(12)
    x = (rng.standard_normal((70_000, 200)) * rng.uniform(0.5, 2.0, (70_000, 1))).astype(np.float32)
    h, st = ctx.hestimate(x, HEST_AMISE)
    assert h.shape == (70_000,) and np.all(h > 0) and np.all(np.isfinite(h))
    assert all(s["conv_evals"] > 0 for s in st[::997])
    pick = [0, 1, 65_534, 65_535, 69_999]
    h5, _ = ctx.hestimate(x, HEST_AMISE, cols=pick)
    assert np.array_equal(h[pick], h5)
