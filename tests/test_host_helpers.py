"""Host-side helpers that need no GPU: the synthetic workloads against the
shapes and distributions of the benchmark configurations, the reference
estimators' host arithmetic (AmiseMin::_amise, hestimate.cpp:41-53;
Tools::sum1_normalized, tools.hxx:33-43; the float log of tools.cpp:29-35)
against the oracle's C restatement, and the autotuner's size buckets and
JSON cache."""
import json

import numpy as np
import pytest

from entropical_gb300 import autotune, estimators, workloads
from oracle import oracle as O


def test_gmm_1d_matches_config():
    x = workloads.gmm_1d(20_000, seed=42)
    assert x.dtype == np.float32 and x.shape == (20_000,)
    # three components at -1.0, 0.2, 1.5 (sd 0.3), weights 0.3 / 0.4 / 0.3
    lo, mid, hi = x < -0.4, (x >= -0.4) & (x < 0.85), x >= 0.85
    assert abs(lo.mean() - 0.3) < 0.02 and abs(mid.mean() - 0.4) < 0.02 and abs(hi.mean() - 0.3) < 0.02
    assert abs(x[lo].mean() + 1.0) < 0.03 and abs(x[hi].mean() - 1.5) < 0.03
    assert np.array_equal(x, workloads.gmm_1d(20_000, seed=42))  # seeded


def test_mi_coords_and_scott():
    x = workloads.mi_coords(5_000, 8, seed=3)
    assert x.dtype == np.float32 and x.shape == (8, 5_000) and x.flags.c_contiguous
    np.testing.assert_allclose(x.mean(axis=1), 0, atol=1e-5)
    np.testing.assert_allclose(x.std(axis=1), 1, atol=1e-5)
    assert np.all(np.abs(np.corrcoef(x)[np.triu_indices(8, 1)]) < 1)  # coupled, not identical
    h = workloads.scott_bandwidth(x, 2)
    np.testing.assert_allclose(h, x.astype(np.float64).std(axis=1) * 5_000 ** (-1 / 6), rtol=1e-6)


def test_langevin_shape_and_coupling():
    x, c = workloads.langevin(n_coords=6, n_steps=2_000, seed=2)
    assert x.dtype == np.float32 and x.shape == (6, 2_000)
    assert np.all(np.diag(c) == 0) and np.all(np.abs(c) <= 0.3)
    assert np.all(np.isfinite(x))


def test_uneven_batch_matches_config():
    b = workloads.uneven_batch(200, seed=5)
    dims = np.array([x.shape[0] for x, _ in b])
    ns = np.array([x.shape[1] for x, _ in b])
    assert set(dims) == {1, 2, 3}
    assert ns.min() >= 2_000 and ns.max() <= 500_000
    # log-uniform sizes: about half below the geometric mean of the range
    assert 0.35 < np.mean(ns < np.sqrt(2_000 * 500_000)) < 0.65
    for x, h in b[:20]:
        assert x.dtype == np.float32 and h.shape == (x.shape[0],) and np.all(h > 0)


def test_amise_formula_matches_oracle():
    rng = np.random.default_rng(1)
    for _ in range(2_000):
        n = int(rng.integers(100, 300_000))
        h = float(np.float32(10 ** rng.uniform(-3, 1)))
        conv = float(np.float32(10 ** rng.uniform(3, 11)))
        a = estimators.amise_from_conv(conv, h, n)
        b = O.amise_from_conv(conv, h, n)
        assert np.float32(a).view(np.uint32) == np.float32(b).view(np.uint32)


def test_sum1_normalized_and_float_log():
    rng = np.random.default_rng(2)
    x = rng.random(10_001) * 10 ** rng.uniform(-8, 8, 10_001)
    y = estimators.sum1_normalized(x)
    assert abs(np.sum(y) - 1.0) < 1e-12
    assert np.array_equal(estimators.sum1_normalized(np.zeros(5)), np.zeros(5))
    v = np.array([0.0, 1.0, 0.5, 1e-30, 3e5], dtype=np.float64)
    lg = estimators._flog(v)
    assert lg.dtype == np.float32 and lg[0] == 0 and lg[1] == 0
    assert np.array_equal(lg[2:], np.log(v[2:].astype(np.float32)))


def test_autotune_buckets_and_cache(tmp_path, monkeypatch):
    assert autotune.bucket(1) == 1 and autotune.bucket(2_000) == 10 and autotune.bucket(2 ** 20) == 20
    cache = tmp_path / "t" / "tuning.json"
    monkeypatch.setenv("ENT_TUNING_CACHE", str(cache))
    assert autotune.cache_path() == cache
    assert autotune._load() == {}
    db = {"GB300|d2|n2^16": {"targets_per_warp": 16, "cells_per_h": 3, "pair_variant": 7, "ms": 4.1}}
    autotune._save(db)
    assert json.loads(cache.read_text()) == db and autotune._load() == db
    cache.write_text("{not json")
    assert autotune._load() == {}  # a damaged cache is ignored


@pytest.mark.parametrize("d", [1, 2, 3])
def test_autotune_candidates_are_supported_shapes(d):
    # every candidate names a body the library builds for that dimension
    for r, s, v in autotune.CANDIDATES[d]:
        assert r in ((8, 16) if d < 3 else (4, 8))
        if v == 6:
            assert d == 1
        if v == 7:
            assert d == 2 and 2 <= s <= 12
