"""Autotuner for the pair-kernel tile shapes.

The persistent pair kernel has three knobs per density dimension d: targets
per warp R (tile = 4 R targets), cells per bandwidth S along dimension 1 of
2-D strips (dimensions 1 and 2 of 3-D strips), and the pair body (0: packed sub/fma + min; 1: saturating FMA;
2: saturating at 5 CTAs/SM; 3: as 2 with larger chunks; 4: symmetric, each
unordered pair once, 4 warps of 32 targets; 5: symmetric, 8 warps of 16;
6, d = 1 only: range sums from exact prefix sums, no pair loop; 7, d = 2
only: strip moments, exact moment prefix sums for the strips inside the
support and pairs only on its edge).
``tune`` times every supported combination on a sample of the caller's own
batch (the first few instances, device time of the pair kernel of that
dimension) and keeps the fastest; results are cached in a JSON file keyed by
device name, dimension and a size bucket, and ``apply`` loads them into a
context.
"""
from __future__ import annotations

import json
import math
import os
from pathlib import Path

from .densities import Context

CANDIDATES = {
    1: [(8, 2, 0), (16, 2, 0), (16, 2, 1), (16, 2, 2), (16, 2, 3), (16, 2, 4), (16, 2, 5),
        (16, 2, 6)],
    2: [(8, 2, 0), (16, 1, 2), (16, 2, 0), (16, 2, 1), (16, 2, 2), (16, 2, 3),
        (16, 1, 4), (16, 2, 4), (16, 2, 5), (16, 3, 7), (16, 4, 7)],
    3: [(4, 1, 0), (8, 1, 0), (8, 1, 1), (8, 1, 2), (8, 2, 2), (8, 1, 3), (8, 1, 4), (8, 2, 4),
        (8, 2, 5)],
}


def _set(ctx: Context, tpw, d: int, s: int, pv) -> None:
    # s: cells per bandwidth of the strips (dimension 1 for d = 2, the strips
    # of the strip-moment body 7, dimensions 1 and 2 for d = 3; unused for
    # d = 1)
    if d == 3:
        ctx.set_tuning(tpw, 0, pv, cells_per_h3=s)
    elif d == 2 and pv[1] == 7:
        ctx.set_tuning(tpw, 0, pv, moment_cells_per_h=s)
    else:
        ctx.set_tuning(tpw, s, pv)


def cache_path() -> Path:
    p = os.environ.get("ENT_TUNING_CACHE")
    if p:
        return Path(p)
    return Path(os.environ.get("XDG_CACHE_HOME", Path.home() / ".cache")) / "entropical_gb300" / "tuning.json"


def _device_name() -> str:
    try:
        import torch
        return torch.cuda.get_device_name(0)
    except Exception:
        return "cuda"


def bucket(n: int) -> int:
    """Size bucket: log2 of the points per instance."""
    return int(math.log2(max(n, 2)))


def _load() -> dict:
    p = cache_path()
    if p.exists():
        try:
            return json.loads(p.read_text())
        except Exception:
            return {}
    return {}


def _save(db: dict) -> None:
    p = cache_path()
    p.parent.mkdir(parents=True, exist_ok=True)
    p.write_text(json.dumps(db, indent=1, sort_keys=True))


def _key(d: int, n: int) -> str:
    return f"{_device_name()}|d{d}|n2^{bucket(n)}"


def tune(ctx: Context, run, d: int, n: int, repeats: int = 2, save: bool = True) -> dict:
    """Time ``run()`` (which must launch instances of dimension d through ctx)
    under every candidate shape; keep and cache the fastest. Returns
    {"targets_per_warp", "cells_per_h", "pair_variant", "ms"}."""
    before = ctx.tuning()
    results = []
    for (r, s, v) in CANDIDATES[d]:
        tpw = list(before["targets_per_warp"])
        tpw[d - 1] = r
        pv = [None, None, None]
        pv[d - 1] = v
        _set(ctx, tpw, d, s, pv)
        run()  # warm-up (all variants are prebuilt)
        best = math.inf
        for _ in range(repeats):
            run()
            best = min(best, ctx.last_stats().pair_kernel_ms_by_dim[d - 1])
        results.append((best, r, s, v))
    best, r, s, v = min(results)
    tpw = list(before["targets_per_warp"])
    tpw[d - 1] = r
    pv = [None, None, None]
    pv[d - 1] = v
    _set(ctx, tpw, d, s, pv)
    choice = {"targets_per_warp": r, "cells_per_h": s, "pair_variant": v, "ms": best,
              "all": [{"r": rr, "s": ss, "v": vv, "ms": mm} for mm, rr, ss, vv in results]}
    if save:
        db = _load()
        db[_key(d, n)] = choice
        _save(db)
    return choice


def apply(ctx: Context, d: int, n: int) -> bool:
    """Load a cached choice for (device, d, size bucket) into ctx; True if found."""
    c = _load().get(_key(d, n))
    if not c:
        return False
    tpw = list(ctx.tuning()["targets_per_warp"])
    tpw[d - 1] = c["targets_per_warp"]
    pv = [None, None, None]
    pv[d - 1] = c["pair_variant"]
    _set(ctx, tpw, d, c["cells_per_h"], pv)
    return True
