"""GPU parity of the batched estimators (one persistent launch for all
instances) against the plain per-instance path and the FP64 oracle.
Entropies and MI: 1e-6 nats absolute against the FP64 oracle; batch vs plain
calls 1e-7 (a small batch splits each tile's sources into a different number
of work items, which changes the FP32 partial sums, not the terms)."""
import numpy as np
import pytest

from entropical_gb300 import workloads
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_mi_all_pairs_matches_oracle(ctx):
    x = workloads.mi_coords(6000, 6, seed=3)
    h = workloads.scott_bandwidth(x, 2)
    mi, hx = ctx.mi_all_pairs(x, h)
    for i in range(6):
        assert abs(hx[i] - O.entropy_fp64(x[i:i + 1], [h[i]])) < 1e-6
    for i, j in [(0, 1), (2, 5), (3, 4)]:
        ref = O.mi_fp64(x[i], x[j], h[i], h[j])
        assert abs(mi[i, j] - ref) < 1e-6
        assert mi[i, j] == mi[j, i]
    assert np.all(np.diag(mi) == 0)


def test_mi_all_pairs_matches_plain_path(ctx):
    x = workloads.mi_coords(20000, 5, seed=8)
    h = workloads.scott_bandwidth(x, 2)
    mi, hx = ctx.mi_all_pairs(x, h)
    for i in range(5):
        p = ctx.combined_densities(x, None, [i], [h[i]])
        assert abs(hx[i] + np.mean(np.log(p))) < 1e-7
    for i, j in [(0, 4), (1, 3)]:
        pij = ctx.combined_densities(x, None, [i, j], [h[i], h[j]])
        assert abs(mi[i, j] - (hx[i] + hx[j] + np.mean(np.log(pij)))) < 1e-7


def test_support_counts_batch(ctx):
    x = workloads.mi_coords(3000, 4, seed=1)
    h = workloads.scott_bandwidth(x, 2)
    cnt, c1 = ctx.mi_all_pairs(x, h, counts=True)
    for i in range(4):
        assert c1[i] == ctx.support_counts(x, None, [i], [h[i]]).sum()
    assert cnt[1, 3] == ctx.support_counts(x, None, [1, 3], [h[1], h[3]]).sum()


def test_uneven_batch(ctx):
    rng = np.random.default_rng(4)
    insts = []
    for q in range(24):
        d = int(rng.integers(1, 4))
        n = int(np.exp(rng.uniform(np.log(50), np.log(30000))))
        x = workloads.mixture_instance(rng, d, n)
        insts.append((x, workloads.scott_bandwidth(x, d)))
    H = ctx.entropy_batch(insts)
    for q in range(0, 24, 3):
        x, h = insts[q]
        assert abs(H[q] - O.entropy_fp64(x, h)) < 1e-6
    # sequential plain calls give the same numbers
    for q in range(1, 24, 5):
        x, h = insts[q]
        p = ctx.combined_densities(x, None, list(range(x.shape[0])), h)
        assert abs(H[q] + np.mean(np.log(p))) < 1e-7


def test_te_all_pairs_matches_oracle(ctx):
    x, _ = workloads.langevin(n_coords=4, n_steps=4000, seed=2)
    h = workloads.scott_bandwidth(x, 3)
    taus = [1, 5]
    te = ctx.te_all_pairs(x, h, taus)
    assert te.shape == (2, 4, 4)
    for q, tau in enumerate(taus):
        for i, j in [(0, 1), (2, 0), (3, 2)]:
            ref = O.te_fp64(x[j], x[i], tau, h[j], h[i])
            assert abs(te[q, i, j] - ref) < 1e-6
        assert np.all(np.diag(te[q]) == 0)


def test_te_support_counts(ctx):
    x, _ = workloads.langevin(n_coords=3, n_steps=2000, seed=3)
    h = workloads.scott_bandwidth(x, 3)
    cnt = ctx.te_all_pairs(x, h, [2], counts=True)
    # 3-D instance (y+, y, x) for i=1, j=2
    c = ctx.support_counts(x, None, [1, 1, 2], [h[1], h[1], h[2]], [2, 0, 0])
    assert cnt[0, 1, 2] == c.sum()


@pytest.mark.parametrize("n_rows,n_cols", [(6000, 5), (100_000, 6)])
def test_mi_split_over_ranks_matches_batch(ctx, n_rows, n_cols):
    """One all-pairs MI dealt over three ranks (run here one after another on
    one GPU, each share one batch from the same device matrix) gives the MI
    batch's numbers; the shares hold every density once. The larger case
    puts the joints on the strip moments."""
    import torch
    from entropical_gb300.replicas import WEIGHTS, deal, mi_assemble, mi_instances
    x = workloads.mi_coords(n_rows, n_cols, seed=21)
    h = workloads.scott_bandwidth(x, 2)
    dx = torch.from_numpy(x).cuda()
    inst = mi_instances(n_cols)
    shares = deal([WEIGHTS[len(c)] for c in inst], 3)
    assert sorted(int(i) for s in shares for i in s) == list(range(len(inst)))
    H = np.zeros(len(inst))
    for items in shares:
        H[items] = ctx.mi_entropies_device(dx.data_ptr(), n_rows, n_cols, h, items)
    mi_s, hx_s = mi_assemble(n_cols, H)
    mi, hx = ctx.mi_all_pairs(x, h)
    assert np.max(np.abs(mi_s - mi)) < 1e-7 and np.max(np.abs(hx_s - hx)) < 1e-7


def test_te_split_over_ranks_matches_batch(ctx):
    """The same for all-ordered-pairs TE at two lags."""
    import torch
    from entropical_gb300.replicas import WEIGHTS, deal, te_assemble, te_instances
    x, _ = workloads.langevin(n_coords=4, n_steps=20_000, seed=8)
    h = workloads.scott_bandwidth(x, 3)
    taus = [1, 7]
    dx = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    inst = te_instances(4, 2)
    dim = {1: 1, 2: 2, 3: 2, 4: 3}
    shares = deal([WEIGHTS[dim[k]] for _, k, _, _ in inst], 3)
    H = np.zeros(len(inst))
    for items in shares:
        H[items] = ctx.te_entropies_device(dx.data_ptr(), x.shape[1], 4, h, taus, items)
    te_s = te_assemble(4, 2, H)
    te = ctx.te_all_pairs(x, h, taus)
    assert np.max(np.abs(te_s - te)) < 1e-7


def test_split_items_errors(ctx):
    import torch
    x = workloads.mi_coords(1000, 3, seed=2)
    h = workloads.scott_bandwidth(x, 2)
    dx = torch.from_numpy(x).cuda()
    with pytest.raises(Exception):
        ctx.mi_entropies_device(dx.data_ptr(), 1000, 3, h, [6])  # 3 + 3 densities: 0..5
    assert len(ctx.mi_entropies_device(dx.data_ptr(), 1000, 3, h, [])) == 0


def test_graph_reuse_across_batches():
    """One context keeps its batch graph: calls alternating between two batch
    shapes (the graph updated in place or instantiated anew) give the same
    numbers as a fresh context for each."""
    from entropical_gb300 import Context
    xa = workloads.mi_coords(8000, 5, seed=31)
    ha = workloads.scott_bandwidth(xa, 2)
    xb = workloads.mi_coords(5000, 7, seed=32)
    hb = workloads.scott_bandwidth(xb, 2)
    with Context(0) as fresh:
        ref_a, _ = fresh.mi_all_pairs(xa, ha)
    with Context(0) as fresh:
        ref_b, _ = fresh.mi_all_pairs(xb, hb)
    with Context(0) as c:
        for _ in range(3):
            mi_a, _ = c.mi_all_pairs(xa, ha)
            mi_b, _ = c.mi_all_pairs(xb, hb)
            assert np.max(np.abs(mi_a - ref_a)) < 1e-9
            assert np.max(np.abs(mi_b - ref_b)) < 1e-9


@pytest.mark.parametrize("d,n", [(1, 30_000), (2, 40_000), (3, 20_000)])
def test_density_target_shares_add_up(ctx, d, n):
    """One density split into target shares (as over GPUs): each share writes
    only its targets; the shares added give the whole density (1e-6 relative
    against the default call, 1e-5 against FP64 at sampled targets) and their
    log sums the entropy."""
    import torch
    x = np.random.default_rng(40 + d).standard_normal((3, n)).astype(np.float32)
    h = [0.3, 0.25, 0.35][:d]
    cols = list(range(d))
    dx = torch.from_numpy(x).cuda()
    total = np.zeros(n)
    ls = 0.0
    for part in range(3):
        buf = torch.zeros(n, dtype=torch.float64, device="cuda")
        n_sel, l = ctx.combined_densities_part_device(dx.data_ptr(), n, 3, cols, h, None, part, 3,
                                                      buf.data_ptr())
        assert n_sel == n
        p = buf.cpu().numpy()
        assert np.all(total[p != 0] == 0)   # each target written by one share
        total += p
        ls += l
    full = ctx.combined_densities(x, None, cols, h)
    assert np.max(np.abs(total - full) / full) < 1e-6
    t = np.random.default_rng(1).choice(n, 500, replace=False)
    f = O.density_fp64(x[:d], h, targets=t)
    assert np.max(np.abs(total[t] - f) / f) < 1e-5
    assert abs(-ls / n - (-np.mean(np.log(full)))) < 1e-9
    with pytest.raises(Exception):
        ctx.combined_densities_part_device(dx.data_ptr(), n, 3, cols, h, None, 3, 3, dx.data_ptr())
