"""The tile-shape autotuner picks a supported shape on the caller's batch,
caches it, and leaves results unchanged."""
import numpy as np
import pytest

from entropical_gb300 import autotune, workloads

pytestmark = pytest.mark.gpu


def test_tune_and_apply(tmp_path, monkeypatch):
    from entropical_gb300 import Context
    monkeypatch.setenv("ENT_TUNING_CACHE", str(tmp_path / "tuning.json"))
    x = workloads.mi_coords(20000, 4, seed=3)
    h = workloads.scott_bandwidth(x, 2)
    with Context(0) as ctx:
        ref, _ = ctx.mi_all_pairs(x, h)
        choice = autotune.tune(ctx, lambda: ctx.mi_all_pairs(x, h), d=2, n=x.shape[1])
        assert (choice["targets_per_warp"], choice["cells_per_h"], choice["pair_variant"]) in \
            [(r, s, v) for r, s, v in autotune.CANDIDATES[2]]
        t = ctx.tuning()
        assert t["pair_variant_by_dim"][1] == choice["pair_variant"]
        mi, _ = ctx.mi_all_pairs(x, h)
        assert np.allclose(mi, ref, atol=1e-5)
    with Context(0) as ctx2:
        assert autotune.apply(ctx2, 2, x.shape[1])
        assert ctx2.tuning()["pair_variant_by_dim"][1] == choice["pair_variant"]


def _cells2(t):
    # the 2-D strip count the chosen body uses
    return t["moment_cells_per_h"] if t["pair_variant_by_dim"][1] == 7 else t["cells_per_h"]


def test_native_autotuner_cache():
    """ent_autotune: the context's own tuner picks a shape per dimension on a
    sample batch, caches it per (d, size bucket), and results stay the same."""
    from entropical_gb300 import Context
    rng = np.random.default_rng(8)
    sample = []
    for d in (1, 2, 3):
        for n in (3000, 7000):
            x = workloads.mixture_instance(rng, d, n)
            sample.append((x, workloads.scott_bandwidth(x, d)))
    with Context(0) as ctx:
        ref = ctx.entropy_batch(sample)
        picks = {}
        for d in (1, 2, 3):
            t = ctx.autotune(sample, d)
            assert 0 <= t["pair_variant_by_dim"][d - 1] <= {1: 6, 2: 7, 3: 5}[d]
            picks[d] = (t["pair_variant_by_dim"][d - 1], _cells2(t), t["cells_per_h3"])
        assert ctx.autotune_cache_size() == 3
        ctx.set_tuning(pair_variant=0, cells_per_h=4, cells_per_h3=2)
        t2 = ctx.autotune(sample, 2)  # cached: applied again without timing
        assert t2["pair_variant_by_dim"][1] == picks[2][0] and _cells2(t2) == picks[2][1]
        assert ctx.autotune_cache_size() == 3
        assert np.allclose(ctx.entropy_batch(sample), ref, rtol=0, atol=2e-6)
