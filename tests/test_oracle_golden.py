"""The CPU oracle against the reference's own outputs (golden fixtures made by
tests/golden/make_golden.py from the reference sources), and -- where the
reference sources are present -- against the live reference build."""
import numpy as np
import pytest

from oracle import oracle as O


def test_density_restatement_bitexact(golden):
    g = golden
    assert np.array_equal(O.density_ref_f32(g["d1_x"], g["d1_h"]), g["d1_p"])
    assert np.array_equal(O.density_ref_f32(g["d2_x"][:2], g["d2_h"]), g["d2_p"])
    assert np.array_equal(O.density_ref_f32(g["d2_x"], g["d3_h"]), g["d3_p"])
    sel = O.repack(g["d2_x"], g["lag_cols"], g["lag_tau"])
    assert np.array_equal(O.density_ref_f32(sel, g["lag_h"]), g["lag_p"])


@pytest.mark.parametrize("case", ["d1", "d2", "d3", "lag"])
def test_fp64_oracle_vs_reference(golden, case):
    g = golden
    if case == "d1":
        sel, h, p = g["d1_x"], g["d1_h"], g["d1_p"]
    elif case == "d2":
        sel, h, p = g["d2_x"][:2], g["d2_h"], g["d2_p"]
    elif case == "d3":
        sel, h, p = g["d2_x"], g["d3_h"], g["d3_p"]
    else:
        sel, h, p = O.repack(g["d2_x"], g["lag_cols"], g["lag_tau"]), g["lag_h"], g["lag_p"]
    f = O.density_fp64(sel, h)
    # the reference accumulates in float32: a few 1e-6 relative
    assert np.max(np.abs(p - f) / f) < 1e-5


def test_boxes_and_boxedsearch(golden):
    g = golden
    lo, hi = O.boxes(g["box_x"], float(g["box_h"][0]))
    assert np.array_equal(lo, g["box_lo"]) and np.array_equal(hi, g["box_hi"])
    nb, _, cnt = O.boxedsearch(g["box_x"], float(g["bs_size"][0]))
    assert nb == int(g["bs_nboxes"][0])
    assert np.array_equal(cnt, g["bs_counts"])


def test_convolution_and_hestimate(golden):
    g = golden
    for h, v in zip(g["conv_h"], g["conv_v"]):
        assert O.epa_conv_ref(g["conv_x"], float(h)) == v
        assert abs(O.epa_conv_fp64(g["conv_x"], float(h)) - v) / v < 1e-6
    for c, t, a in zip(g["hest_x"], g["hest_thumb"], g["hest_amise"]):
        assert O.thumb_ref(c) == t
        h, ncalls = O.hestimate_amise(c, exact=True)
        assert h == a and ncalls == 16
        assert O.hestimate_amise(c, exact=False)[0] == a


def test_amise_search_takes_top_leaf(golden):
    # The reference objective (hestimate.cpp:41-53) decreases monotonically in h,
    # so the bisection always keeps the upper half: h = 2 h0 - 1.9 h0 / 512.
    r = golden["hest_amise"] / golden["hest_thumb"]
    assert np.allclose(r, 2 - 1.9 / 512, rtol=1e-6)


live = pytest.mark.skipif(not O.ref_available(), reason="reference build not present")


@live
@pytest.mark.parametrize("d", [1, 2, 3])
def test_live_reference_random(d):
    rng = np.random.default_rng(100 + d)
    x = rng.standard_normal((3, 2500)).astype(np.float32)
    h = rng.uniform(0.1, 0.5, d).astype(np.float32)
    cols = list(rng.permutation(3)[:d])
    tau = list(rng.integers(0, 9, d))
    p = O.ref_densities(x, cols, h, tau)
    assert np.array_equal(O.density_ref_f32(O.repack(x, cols, tau), h), p)


@live
def test_live_reference_boxes_ties():
    rng = np.random.default_rng(5)
    col = np.round(rng.standard_normal(2000) * 20).astype(np.float32) / 20
    lo, hi = O.ref_boxes(col, 0.1)
    lo2, hi2 = O.boxes(col, 0.1)
    assert np.array_equal(lo, lo2) and np.array_equal(hi, hi2)


@pytest.mark.parametrize("name,key,tau", [("mi", "est_mi", 0), ("transs", "est_transs", 2),
                                          ("autoent", "est_autoent", 2), ("negs", "est_negs", 0),
                                          ("kldiv", "est_kldiv", 0)])
def test_reference_estimator_formulas_vs_golden(golden, name, key, tau):
    """The FP64 restatement of the reference estimator formulas reproduces the
    reference's own estimator outputs (printed to 6 significant digits)."""
    r = O.reference_estimator_fp64(golden["est_x"], golden["est_h"], name, tau)
    g = golden[key].reshape(r.shape)
    assert np.allclose(r, g, rtol=2e-5, atol=1e-6)
