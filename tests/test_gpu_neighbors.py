"""Neighbour searches on the GPU are bit-exact with the reference's boxes()
windows and BoxedSearch neighbour lists."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_windows_golden(ctx, golden):
    lo, hi = ctx.neighbor_windows(golden["box_x"], float(golden["box_h"][0]))
    assert np.array_equal(lo, golden["box_lo"]) and np.array_equal(hi, golden["box_hi"])


def test_boxed_golden(ctx, golden):
    nb, _, cnt = ctx.boxed_neighbors(golden["box_x"], float(golden["bs_size"][0]))
    assert nb == int(golden["bs_nboxes"][0])
    assert np.array_equal(cnt, golden["bs_counts"])


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_windows_random_with_ties(ctx, seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 200_000))
    x = (np.round(rng.standard_normal(n) * 50) / 50).astype(np.float32)
    h = float(rng.uniform(0.001, 0.5))
    lo, hi = ctx.neighbor_windows(x, h)
    lo2, hi2 = O.boxes(x, h)
    assert np.array_equal(lo, lo2) and np.array_equal(hi, hi2)


def test_boxed_edge_cases(ctx):
    # integer range/box ratio (index == box count in the reference) and a
    # constant column (zero boxes in the reference)
    x = np.array([0.0, 0.5, 1.0, 1.5, 2.0], np.float32)
    nb, box, cnt = ctx.boxed_neighbors(x, 0.5)
    nb2, box2, cnt2 = O.boxedsearch(x, 0.5)
    assert nb == nb2 and np.array_equal(box, box2) and np.array_equal(cnt, cnt2)
    x = np.full(7, 3.0, np.float32)
    nb, box, cnt = ctx.boxed_neighbors(x, 0.1)
    assert nb == 1 and np.all(cnt == 7)
