"""The reference estimators' own formulas over GPU densities reproduce the
outputs of the reference's estimator mains (golden fixtures; the reference
prints 6 significant digits)."""
import numpy as np
import pytest

from entropical_gb300.estimators import ReferenceEstimators

pytestmark = pytest.mark.gpu


def close(a, b, rtol=2e-5, atol=1e-6):
    return np.allclose(np.asarray(a, np.float64), np.asarray(b, np.float64), rtol=rtol, atol=atol)


def test_mi(ctx, golden):
    est = ReferenceEstimators(ctx)
    assert close(est.mi(golden["est_x"], golden["est_h"]), golden["est_mi"])


def test_transs(ctx, golden):
    est = ReferenceEstimators(ctx)
    assert close(est.transs(golden["est_x"], golden["est_h"], 2), golden["est_transs"])


def test_autoent_negs_kldiv(ctx, golden):
    est = ReferenceEstimators(ctx)
    assert close(est.autoent(golden["est_x"], golden["est_h"], 2), golden["est_autoent"])
    assert close(est.negs(golden["est_x"], golden["est_h"]), golden["est_negs"])
    assert close(est.kldiv(golden["est_x"], golden["est_h"]), golden["est_kldiv"])


def test_dens_pairs(ctx, golden):
    est = ReferenceEstimators(ctx)
    assert close(est.dens_nd(golden["est_x"], golden["est_h"], 2), golden["est_dens2"], rtol=1e-4)


def test_plain_amise_loop_matches_batched_search(ctx, golden):
    from entropical_gb300.densities import HEST_AMISE, HEST_THUMB
    from entropical_gb300.estimators import hestimate_amise_plain
    h0, _ = ctx.hestimate(golden["hest_x"], HEST_THUMB)
    hb, _ = ctx.hestimate(golden["hest_x"], HEST_AMISE)
    for c, t, ref in zip(golden["hest_x"], h0, golden["hest_amise"]):
        h, calls = hestimate_amise_plain(ctx, c, t)
        assert calls == 16
        assert np.float32(h) == ref
    assert np.array_equal(hb, golden["hest_amise"])


def test_dens_triples(ctx, golden):
    est = ReferenceEstimators(ctx)
    assert close(est.dens_nd(golden["est_x"], golden["est_h"], 3), golden["est_dens3"], rtol=1e-4)
