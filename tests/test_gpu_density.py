"""GPU parity of the density path: the CUDA library (through the C ABI)
against the reference's golden outputs and the FP64 oracle.

Tolerance: densities 1e-5 relative per point (the reference itself is a
float32 accumulation, ~3e-6 from FP64); support counts and entropies
derived from them as stated per test."""
import numpy as np
import pytest

from entropical_gb300 import NativeError, workloads
from oracle import oracle as O

pytestmark = pytest.mark.gpu

REL = 1e-5


def rel_err(a, b):
    return np.max(np.abs(np.asarray(a) - np.asarray(b)) / np.abs(np.asarray(b)))


@pytest.mark.parametrize("case", ["d1", "d2", "d3", "lag"])
def test_golden_reference(ctx, golden, case):
    g = golden
    if case == "d1":
        p = ctx.combined_densities(g["d1_x"], None, [0], g["d1_h"])
        ref = g["d1_p"]
    elif case == "d2":
        p = ctx.combined_densities(g["d2_x"], None, [0, 1], g["d2_h"])
        ref = g["d2_p"]
    elif case == "d3":
        p = ctx.combined_densities(g["d2_x"], None, [0, 1, 2], g["d3_h"])
        ref = g["d3_p"]
    else:
        p = ctx.combined_densities(g["d2_x"], None, list(g["lag_cols"]), g["lag_h"],
                                   list(g["lag_tau"]))
        ref = g["lag_p"]
    assert p.shape == ref.shape
    assert rel_err(p, ref) < REL


@pytest.mark.parametrize("d", [1, 2, 3])
@pytest.mark.parametrize("n", [1, 2, 33, 1000, 20000])
def test_fp64_oracle_shapes(ctx, d, n):
    rng = np.random.default_rng(1000 * d + n)
    x = rng.standard_normal((3, n)).astype(np.float32)
    h = rng.uniform(0.15, 0.6, d).astype(np.float32)
    cols = list(rng.permutation(3)[:d])
    p = ctx.combined_densities(x, None, cols, h)
    f = O.density_fp64(O.repack(x, cols), h)
    assert rel_err(p, f) < REL


@pytest.mark.parametrize("d", [1, 2, 3])
def test_lags_and_compat_norm(ctx, d):
    rng = np.random.default_rng(77 + d)
    x = rng.standard_normal((4, 3000)).astype(np.float32)
    cols = [1, 1, 3][:d]
    tau = [0, 11, 4][:d]
    h = [0.3, 0.25, 0.4][:d]
    sel = O.repack(x, cols, tau)
    p = ctx.combined_densities(x, None, cols, h, tau)
    assert len(p) == 3000 - max(tau)
    assert rel_err(p, O.density_fp64(sel, h)) < REL
    pc = ctx.combined_densities(x, None, cols, h, tau, compat_norm=True)
    assert rel_err(pc, O.density_fp64(sel, h, norm=3000)) < REL


@pytest.mark.parametrize("d", [1, 2, 3])
def test_edge_data(ctx, d):
    rng = np.random.default_rng(9)
    n = 4000
    # exact ties, a constant column, negative-only values, a far outlier
    x = np.stack([
        np.round(rng.standard_normal(n) * 4) / 4,
        np.full(n, -3.0),
        -np.abs(rng.standard_normal(n)) - 1.0,
    ]).astype(np.float32)
    x[0, 17] = 1e4
    h = [0.2, 0.5, 0.3][:d]
    for cols in ([0, 1, 2][:d], [2, 0, 1][:d]):
        p = ctx.combined_densities(x, None, cols, h)
        assert rel_err(p, O.density_fp64(O.repack(x, cols), h)) < REL


@pytest.mark.parametrize("d", [1, 2, 3])
def test_tiny_and_huge_bandwidth(ctx, d):
    rng = np.random.default_rng(3)
    x = rng.standard_normal((3, 3000)).astype(np.float32)
    cols = [0, 1, 2][:d]
    for hv in (1e-6, 50.0):
        h = [hv] * d
        p = ctx.combined_densities(x, None, cols, h)
        assert rel_err(p, O.density_fp64(O.repack(x, cols), h)) < REL


@pytest.mark.parametrize("d", [1, 2, 3])
def test_support_counts_exact(ctx, d):
    rng = np.random.default_rng(40 + d)
    n = 1500
    x = rng.standard_normal((3, n)).astype(np.float32)
    h = np.array([0.3, 0.4, 0.5][:d], np.float32)
    cols = [0, 1, 2][:d]
    c = ctx.support_counts(x, None, cols, h)
    # brute force with the kernel's own test: coordinates scaled by the exact
    # power of two 2^k (g = h 2^k in [1, 2)), fma(d, d, -g^2) <= 0, which
    # equals d*d <= g^2 in exact arithmetic
    inside = np.ones((n, n), bool)
    for j, c_ in enumerate(cols):
        k = 1 - np.frexp(np.float32(h[j]))[1]
        sc = np.float32(2.0 ** k)
        g = np.float32(h[j]) * sc
        y = x[c_] * sc
        dd = (y[:, None] - y[None, :]).astype(np.float64)
        inside &= dd * dd <= np.float64(np.float32(g * g))
    assert np.array_equal(c, inside.sum(1).astype(np.float64))


def test_device_pointer_form(ctx):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(2)
    x = rng.standard_normal((2, 5000)).astype(np.float32)
    dx = torch.from_numpy(x).cuda()
    dout = torch.empty(5000, dtype=torch.float64, device="cuda")
    n = ctx.combined_densities_device(dx.data_ptr(), 5000, 2, [0, 1], [0.3, 0.3], None,
                                      dout.data_ptr())
    torch.cuda.synchronize()
    assert n == 5000
    p = dout.cpu().numpy()
    assert rel_err(p, ctx.combined_densities(x, None, [0, 1], [0.3, 0.3])) < 1e-12


def test_errors_are_status_codes(ctx):
    x = np.zeros((2, 10), np.float32)
    with pytest.raises(NativeError) as e:
        ctx.combined_densities(x, None, [], [])
    assert e.value.status == 1
    with pytest.raises(NativeError) as e:
        ctx.combined_densities(x, None, [0, 1, 0, 1], [1, 1, 1, 1])
    assert e.value.status == 1
    with pytest.raises(NativeError) as e:
        ctx.combined_densities(x, None, [0], [1.0, 2.0])
    assert e.value.status == 2
    with pytest.raises(NativeError) as e:
        ctx.combined_densities(x, None, [0], [-1.0])
    assert e.value.status == 4
    with pytest.raises(NativeError) as e:
        ctx.combined_densities(x, None, [5], [1.0])
    assert e.value.status == 4
    with pytest.raises(NativeError) as e:
        ctx.combined_densities(x, None, [0], [1.0], [10])
    assert e.value.status == 4
    y = x.copy()
    y[0, 3] = np.nan
    with pytest.raises(NativeError) as e:
        ctx.combined_densities(y, None, [0], [1.0])
    assert e.value.status == 5
    # the context stays usable after errors
    assert ctx.combined_densities(x + 1, None, [0], [1.0]).shape == (10,)


def test_config1_full_size(ctx):
    x = workloads.gmm_1d(20_000, seed=42)[None]
    p = ctx.combined_densities(x, None, [0], [0.1])
    f = O.density_fp64(x, [0.1])
    assert rel_err(p, f) < REL
    H = -np.mean(np.log(p))
    Hf = -np.mean(np.log(f))
    assert abs(H - Hf) < 1e-6


def test_mi_config_pair_sampled(ctx):
    x = workloads.mi_coords(100_000, 8, seed=2024)
    h = workloads.scott_bandwidth(x, 2)
    p = ctx.combined_densities(x, None, [2, 5], [h[2], h[5]])
    t = np.random.default_rng(0).choice(100_000, 3000, replace=False)
    f = O.density_fp64(O.repack(x, [2, 5]), [h[2], h[5]], targets=t)
    assert rel_err(p[t], f) < REL


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
@pytest.mark.parametrize("d", [1, 2, 3])
def test_pair_body_variants(d, variant):
    from entropical_gb300 import Context
    rng = np.random.default_rng(60 + d)
    x = rng.standard_normal((3, 6000)).astype(np.float32)
    h = [0.2, 0.3, 0.25][:d]
    cols = [2, 0, 1][:d]
    with Context(0) as c:
        c.set_tuning(pair_variant=variant)
        assert c.tuning()["pair_variant"] == variant
        p = c.combined_densities(x, None, cols, h)
        assert rel_err(p, O.density_fp64(O.repack(x, cols), h)) < REL
        for hv in (1e-6, 50.0):
            p = c.combined_densities(x, None, cols, [hv] * d)
            assert rel_err(p, O.density_fp64(O.repack(x, cols), [hv] * d)) < REL


def test_epilogue_log(ctx):
    """The table-reduction FP64 log of the per-point epilogues is within
    5e-16 * max(1, |log x|) of the FP64 log (absolute accuracy is what the
    entropy sums need); non-normal inputs take the library log."""
    rng = np.random.default_rng(12)
    x = np.concatenate([10 ** rng.uniform(-300, 300, 100_000), 10 ** rng.uniform(-9, 4, 100_000),
                        1 + rng.uniform(-1e-3, 1e-3, 5000), 0.5 + rng.uniform(-1e-3, 1e-3, 5000),
                        2.0 ** np.arange(-1000, 1000, 7), [1.0, 2.0, 0.5, np.nextafter(1, 2)]])
    y = ctx.log64_selftest(x)
    ref = np.log(x)
    assert np.all(np.abs(y - ref) <= 5e-16 * np.maximum(1.0, np.abs(ref)))
    special = np.array([5e-324, 1e-310, np.inf, 0.0])
    with np.errstate(divide="ignore"):
        assert np.allclose(ctx.log64_selftest(special)[:3], np.log(special[:3]), rtol=1e-15)
    assert ctx.log64_selftest(special)[3] == -np.inf


def test_bounded_wait_reports_timeout():
    """A device-side wait that nothing completes gives up after its bound; the
    call returns ENT_ERR_TIMEOUT and the context keeps working."""
    import time
    from entropical_gb300 import Context
    with Context(0) as c:
        t0 = time.perf_counter()
        st = c.lib.ent_wait_selftest(c.handle)
        dt = time.perf_counter() - t0
        assert st == 8, st  # ENT_ERR_TIMEOUT
        assert 1.5 < dt < 30
        x = np.random.default_rng(3).standard_normal((2, 2000)).astype(np.float32)
        p = c.combined_densities(x, None, [0, 1], [0.3, 0.3])
        assert rel_err(p, O.density_fp64(x, [0.3, 0.3])) < REL


def test_integer_log_of_exact_sums(ctx):
    """The strip-moment epilogue's log of an exact 128-bit sum, in 2^-48 fixed
    point, against a 40-digit decimal log: within 2^-45 (2.9e-14) absolute."""
    from decimal import Decimal, getcontext
    getcontext().prec = 40
    rng = np.random.default_rng(17)
    vals = [1, 2, 3, 2 ** 47, 2 ** 47 + 1, 2 ** 92, 3 * 2 ** 90, 2 ** 127 - 1, 2 ** 64 - 1,
            2 ** 64, 10 ** 30]
    for bits in (20, 47, 48, 60, 64, 80, 92, 100, 110, 120, 127):
        vals += [int(rng.integers(1 << 30)) << max(0, bits - 30) | int(rng.integers(1 << 20))
                 for _ in range(40)]
    # values right at the table's cell edges (top 8 bits after the leading one)
    for k in range(0, 256, 5):
        vals.append((256 + k) << 84)
        vals.append(((256 + k) << 84) - 1)
    out = ctx.ilog_selftest(vals)
    for v, o in zip(vals, out):
        ref = Decimal(v).ln() * (Decimal(2) ** 48)
        assert abs(Decimal(int(o)) - ref) <= 8, (v, int(o), ref)  # 2^-45
