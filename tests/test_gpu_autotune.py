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
