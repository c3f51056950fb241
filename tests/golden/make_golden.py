"""Generate tests/golden/reference_golden.npz from the reference's own code.

The reference (lettis/entropical) ships no tests or golden vectors, so the
fixtures are produced by running its OpenMP sources, compiled in place by
``make -C oracle ref`` (needs the reference checkout: ``--reference``,
$ENT_REFERENCE, or a ``reference`` directory beside this repository), on
small seeded inputs. The committed fixtures let the
oracle and the CUDA path be checked against the reference on machines where
the reference sources are absent.

Usage:  python tests/golden/make_golden.py [--reference PATH]
"""
from __future__ import annotations

import argparse
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from entropical_gb300 import workloads  # noqa: E402
from oracle import oracle as O  # noqa: E402


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None,
                    help="reference checkout (default: $ENT_REFERENCE or ../reference)")
    args = ap.parse_args()
    if O.build_ref(args.reference) is None:
        raise SystemExit("reference sources not found")
    O.build_oracle()
    rng = np.random.default_rng(20261203)
    g: dict[str, np.ndarray] = {}

    # 1-D density on the config-1 mixture (smaller N) and continuous 2-D/3-D data
    x1 = workloads.gmm_1d(2000, seed=7)
    g["d1_x"] = x1[None]
    g["d1_h"] = np.array([0.1], np.float32)
    g["d1_p"] = O.ref_densities(g["d1_x"], [0], g["d1_h"])

    x2 = rng.standard_normal((3, 1500)).astype(np.float32)
    x2[1] = 0.6 * x2[0] + 0.8 * x2[1]
    g["d2_x"] = x2
    g["d2_h"] = np.array([0.25, 0.3], np.float32)
    g["d2_p"] = O.ref_densities(x2, [0, 1], g["d2_h"])
    g["d3_h"] = np.array([0.4, 0.35, 0.5], np.float32)
    g["d3_p"] = O.ref_densities(x2, [0, 1, 2], g["d3_h"])
    # lagged, repeated and permuted selections (transs.cpp:137-146 style)
    g["lag_cols"] = np.array([2, 2, 0], np.uint32)
    g["lag_tau"] = np.array([0, 7, 0], np.uint32)
    g["lag_h"] = np.array([0.5, 0.5, 0.4], np.float32)
    g["lag_p"] = O.ref_densities(x2, g["lag_cols"], g["lag_h"], g["lag_tau"])

    # boxes() windows and Transs::BoxedSearch neighbour counts
    col = (rng.standard_normal(3000) * 0.7 + 0.3).astype(np.float32)
    g["box_x"] = col
    g["box_h"] = np.array([0.05], np.float32)
    lo, hi = O.ref_boxes(col, 0.05)
    g["box_lo"], g["box_hi"] = lo, hi
    g["bs_size"] = np.array([0.13], np.float32)
    nb, cnt = O.ref_boxedsearch(col, 0.13)
    g["bs_nboxes"] = np.array([nb], np.uint64)
    g["bs_counts"] = cnt

    # AMISE convolution, Thumb and the full AMISE bandwidth search
    cs = np.sort(workloads.gmm_1d(1200, seed=9))
    g["conv_x"] = cs
    g["conv_h"] = np.array([0.05, 0.2, 0.9], np.float32)
    g["conv_v"] = np.array([O.ref_epa_convolution(cs, float(h)) for h in g["conv_h"]], np.float32)
    hcols = np.stack([workloads.mixture_instance(np.random.default_rng(s), 1, 900)[0]
                      for s in (1, 2, 3)])
    g["hest_x"] = hcols
    g["hest_thumb"] = np.array([O.ref_thumb(c) for c in hcols], np.float32)
    g["hest_amise"] = np.array([O.ref_amise_h(c) for c in hcols], np.float32)

    # estimator modes through their own main() functions (CUDA-build signature)
    est = rng.standard_normal((4, 600)).astype(np.float32)
    est[1] = 0.7 * est[0] + 0.5 * est[1]
    est[3] = np.roll(est[2], 2) * 0.8 + 0.3 * est[3]
    bw = np.array([0.4, 0.35, 0.45, 0.5], np.float32)
    g["est_x"], g["est_h"] = est, bw
    with tempfile.TemporaryDirectory() as td:
        g["est_mi"] = O.ref_run_mode("mi", est, bw, Path(td) / "mi")
        g["est_transs"] = O.ref_run_mode("transs", est, bw, Path(td) / "te", tau=2)
        g["est_autoent"] = O.ref_run_mode("autoent", est, bw, Path(td) / "ae", tau=2).ravel()
        g["est_negs"] = O.ref_run_mode("negs", est, bw, Path(td) / "ng").ravel()
        g["est_kldiv"] = O.ref_run_mode("kldiv", est, bw, Path(td) / "kl")
        g["est_dens2"] = O.ref_run_mode("dens", est, bw, Path(td) / "d2", dims=2)
        g["est_dens3"] = O.ref_run_mode("dens", est, bw, Path(td) / "d3", dims=3)
    out = ROOT / "tests" / "golden" / "reference_golden.npz"
    np.savez_compressed(out, **g)
    print("wrote", out, out.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
