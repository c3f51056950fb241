"""The reference estimators' own formulas over GPU densities reproduce the
outputs of the reference's estimator mains (golden fixtures; the reference
prints 6 significant digits), both as one device batch each
(ent_reference_estimator / ent_dens_all, the default) and in the reference's
per-density loop structure (batched=False); the device batches also match
the FP64 oracle of the same formulas (within 1e-6 of sum_k |term| + |weight|:
float logs of FP32-summed densities, FP64 sums)."""
import numpy as np
import pytest

from entropical_gb300 import workloads
from entropical_gb300.estimators import ReferenceEstimators
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def close(a, b, rtol=2e-5, atol=1e-6):
    return np.allclose(np.asarray(a, np.float64), np.asarray(b, np.float64), rtol=rtol, atol=atol)


@pytest.fixture(params=[True, False], ids=["batched", "per_call"])
def est(ctx, request):
    return ReferenceEstimators(ctx, batched=request.param)


def test_mi(est, golden):
    assert close(est.mi(golden["est_x"], golden["est_h"]), golden["est_mi"])


def test_transs(est, golden):
    assert close(est.transs(golden["est_x"], golden["est_h"], 2), golden["est_transs"])


def test_autoent_negs_kldiv(est, golden):
    assert close(est.autoent(golden["est_x"], golden["est_h"], 2), golden["est_autoent"])
    assert close(est.negs(golden["est_x"], golden["est_h"]), golden["est_negs"])
    assert close(est.kldiv(golden["est_x"], golden["est_h"]), golden["est_kldiv"])


def test_dens_pairs(est, golden):
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


def test_dens_triples(est, golden):
    assert close(est.dens_nd(golden["est_x"], golden["est_h"], 3), golden["est_dens3"], rtol=1e-4)


@pytest.mark.parametrize("name,kind,tau", [("mi", 1, 0), ("transs", 2, 3), ("autoent", 3, 5),
                                           ("negs", 4, 0), ("kldiv", 5, 0)])
def test_device_estimators_vs_fp64_oracle(ctx, name, kind, tau):
    x = workloads.mi_coords(4000, 5, seed=31)
    h = workloads.scott_bandwidth(x, 2)
    r = ctx.reference_estimator(x, h, kind, tau)
    f, bnd = O.reference_estimator_fp64(x, h, name, tau, bound=True)
    # FP32-summed densities (<= 1e-6 relative) under float logs: the error
    # scale of each output is sum_k (|term| + |weight|)
    assert np.all(np.abs(r - f) <= 1e-6 * bnd + 1e-12)
    # sums run one block per output in a fixed order; only the FP64 atomic
    # order inside the densities varies between calls
    assert np.allclose(r, ctx.reference_estimator(x, h, kind, tau), rtol=1e-12, atol=1e-15)


def test_dens_all_vs_oracle(ctx):
    x = workloads.mi_coords(3000, 4, seed=5)
    h = workloads.scott_bandwidth(x, 2)
    d1 = ctx.dens_all(x, h, 1)
    assert d1.shape == (4, 3000)
    for i in range(4):
        p = O.density_fp64(x[i:i + 1], [h[i]])
        assert np.max(np.abs(d1[i] - p / p.sum()) / (p / p.sum())) < 1e-5
    d3 = ctx.dens_all(x, h, 3, [0, 2, 1])
    assert d3.shape == (4, 2998)
    for r, (i, j, k) in enumerate([(0, 1, 2), (0, 1, 3), (0, 2, 3), (1, 2, 3)]):
        sel = np.stack([x[i][0:2998], x[j][2:3000], x[k][1:2999]])
        p = O.density_fp64(sel, [h[i], h[j], h[k]])
        assert np.max(np.abs(d3[r] - p / p.sum()) / (p / p.sum())) < 1e-5
    assert np.allclose(d3.sum(1), 1.0, rtol=1e-12)


def test_estimator_argument_errors(ctx):
    from entropical_gb300 import NativeError
    x = np.zeros((2, 10), np.float32)
    with pytest.raises(NativeError):
        ctx.reference_estimator(x, [0.1, 0.1], 9)
    with pytest.raises(NativeError):
        ctx.reference_estimator(x, [0.1, 0.1], 2, tau=10)
    with pytest.raises(NativeError):
        ctx.reference_estimator(x, [0.1, -1.0], 1)
    with pytest.raises(NativeError):
        ctx.dens_all(x, [0.1, 0.1], 4)


def test_device_input_and_output_forms(ctx):
    torch = pytest.importorskip("torch")
    x = workloads.mi_coords(3000, 4, seed=9)
    h = workloads.scott_bandwidth(x, 2)
    dx = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    for kind, tau in ((1, 0), (2, 2), (3, 3), (4, 0), (5, 0)):
        r_dev = ctx.reference_estimator_device(dx.data_ptr(), 3000, 4, h, kind, tau)
        assert np.allclose(r_dev, ctx.reference_estimator(x, h, kind, tau), rtol=1e-12, atol=1e-15)
    out = torch.zeros((4, 2999), dtype=torch.float64, device="cuda")
    ni, ns = ctx.dens_all_device(dx.data_ptr(), 3000, 4, h, 3, out.data_ptr(), [0, 1, 0])
    torch.cuda.synchronize()
    assert (ni, ns) == (4, 2999)
    assert np.allclose(out.cpu().numpy(), ctx.dens_all(x, h, 3, [0, 1, 0]), rtol=1e-12, atol=0)
