"""Degenerate shapes through the batched entry points: one column, one row,
empty batches, lags at the limit. Results against the FP64 oracle where they
are defined, status codes where the reference would reject the input."""
import numpy as np
import pytest

from entropical_gb300 import NativeError
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_single_column_batches(ctx):
    x = np.random.default_rng(0).standard_normal((1, 500)).astype(np.float32)
    mi, hx = ctx.mi_all_pairs(x, [0.3])
    assert mi.shape == (1, 1) and mi[0, 0] == 0
    assert abs(hx[0] - O.entropy_fp64(x, [0.3])) < 1e-6
    te = ctx.te_all_pairs(x, [0.3], [1])
    assert te.shape == (1, 1, 1) and te[0, 0, 0] == 0
    assert np.array_equal(ctx.reference_estimator(x, [0.3], 1), np.zeros((1, 1)))
    negs = ctx.reference_estimator(x, [0.3], 4)
    assert np.allclose(negs, O.reference_estimator_fp64(x, [0.3], "negs"), rtol=1e-6)
    assert ctx.dens_all(x, [0.3], 2).shape == (0, 500)
    assert ctx.dens_all(x, [0.3], 1).shape == (1, 500)


def test_empty_batch_and_single_points(ctx):
    assert ctx.entropy_batch([]).shape == (0,)
    x1 = np.array([[0.25]], np.float32)
    p = ctx.combined_densities(x1, None, [0], [0.25])  # h exact in float
    assert np.allclose(p, [0.75 / 0.25], rtol=1e-7)
    z = np.zeros((3, 1), np.float32)
    mi, hx = ctx.mi_all_pairs(z, [0.25] * 3)
    assert np.allclose(hx, -np.log(0.75 / 0.25), rtol=1e-12)
    assert np.allclose(mi, 0.0, atol=1e-12)


def test_lag_limits(ctx):
    x = np.random.default_rng(1).standard_normal((2, 50)).astype(np.float32)
    with pytest.raises(NativeError) as e:
        ctx.te_all_pairs(x, [0.3, 0.3], [50])
    assert e.value.status == 4
    te = ctx.te_all_pairs(x, [0.3, 0.3], [49])  # one sample left
    assert np.all(np.isfinite(te))
    r = ctx.reference_estimator(x[:, :3], [0.3, 0.3], 2, 2)
    assert np.all(np.isfinite(r))
    with pytest.raises(NativeError):
        ctx.reference_estimator(x, [0.3, 0.3], 3, 50)
