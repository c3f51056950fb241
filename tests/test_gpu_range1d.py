"""GPU parity of the 1-D range-sum body (pair_variant_by_dim[0] = 6, the
default for d = 1): every target's support is one range of the value-sorted
points and its density comes from exact fixed-point prefix sums.

Checked against the FP64 oracle at 1e-5 relative per point (the plain-path
bar), and against the symmetric pair body at 1e-6 relative (the two differ
only by FP32 rounding in the pair loop), on data chosen to break prefix sums
taken in floating point: a large offset, heavy ties, extreme outliers, a
spread far below the bandwidth, and a bandwidth so small that only the
point itself is in its support. Entropies 1e-6 nats against FP64."""
import numpy as np
import pytest

from entropical_gb300 import workloads
from oracle import oracle as O

pytestmark = pytest.mark.gpu

REL = 1e-5


def rel_err(a, b):
    return np.max(np.abs(np.asarray(a) - np.asarray(b)) / np.abs(np.asarray(b)))


def _cases():
    rng = np.random.default_rng(77)
    g = workloads.gmm_1d(20000, seed=7)
    return {
        "gmm": (g, 0.1),
        "offset": (g + np.float32(1000.0), 0.05),
        "ties": (np.round(g, 2).astype(np.float32), 0.03),
        "outliers": (np.concatenate([g[:5000], np.float32([1e30, -3e25, 7e20])]), 0.08),
        "narrow": (rng.normal(5.0, 1e-4, 3000).astype(np.float32), 0.5),
        "self_only": (np.arange(500, dtype=np.float32) * np.float32(0.37), 0.1),
        "tiny_n": (np.float32([0.3, -1.2]), 1.0),
        "one": (np.float32([2.5]), 0.2),
    }


@pytest.mark.parametrize("name", list(_cases()))
def test_range_fp64(ctx, name):
    assert ctx.tuning()["pair_variant_by_dim"][0] == 6
    x, h = _cases()[name]
    p = ctx.combined_densities(x[None, :], None, [0], [h])
    ref = O.density_fp64(x[None, :], [h])
    assert rel_err(p, ref) < REL


@pytest.mark.parametrize("name", ["gmm", "offset", "ties", "outliers"])
def test_range_vs_symmetric_pair_body(name):
    from entropical_gb300 import Context
    x, h = _cases()[name]
    with Context(0) as a, Context(0) as b:
        b.set_tuning(pair_variant=[4, None, None])
        assert b.tuning()["pair_variant_by_dim"][0] == 4
        pa = a.combined_densities(x[None, :], None, [0], [h])
        pb = b.combined_densities(x[None, :], None, [0], [h])
    assert rel_err(pa, pb) < 1e-6


def test_range_entropy_and_batch(ctx):
    rng = np.random.default_rng(5)
    items = [(workloads.mixture_instance(rng, 1, n)[0][None, :], np.float32([hh]))
             for n, hh in [(3000, 0.05), (17, 0.4), (9000, 0.2), (2, 0.7)]]
    H = ctx.entropy_batch(items)
    for q, (x, h) in enumerate(items):
        assert abs(H[q] - O.entropy_fp64(x, h)) < 1e-6
    # the batch and the single-instance path give the same entropies
    for q, (x, h) in enumerate(items):
        p = ctx.combined_densities(x, None, [0], h)
        assert abs(H[q] + np.mean(np.log(p))) < 1e-9


def test_range_counts_use_pair_body(ctx):
    x, h = _cases()["ties"]
    c = ctx.entropy_batch([(x[None, :], np.float32([h]))], counts=True)[0]
    assert c == O.support_count_fp64(x[None, :], [h])


def test_range_variant_only_for_one_dimension(ctx):
    from entropical_gb300._native import NativeError
    with pytest.raises(NativeError):
        ctx.set_tuning(pair_variant=[None, 6, None])
    with pytest.raises(NativeError):
        ctx.set_tuning(pair_variant=6)
