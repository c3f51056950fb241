#!/usr/bin/env python3
"""Benchmark of the entropical GB300 density hot path.

Workload (one step): all-pairs mutual information over 64 coordinates x
100,000 frames -- 64 1-D marginal densities and 2,016 2-D joint densities,
Scott-rule bandwidths, resubstitution MI -- computed as ONE batch through the
library (1-D range sums and 2-D strip moments by default, one launch
sequence per dimension). Synthetic, seeded data: x_t = tanh(A z_t), z a
16-dim AR(1) (phi 0.95), columns standardised.

value      in-support pair-kernel evaluations per second (the step's work in
           the reference's unit), inputs resident in HBM
           (ent_mi_all_pairs_device), device time on the library stream
e2e        same metric through the host-buffer C-ABI call ent_mi_all_pairs,
           host->device copy of the coordinates and device->host copy of the
           MI matrix inside the timed region
roofline   the dominant 2-D kernels: for the strip moments, compulsory HBM
           bytes over their time against the measured copy bandwidth (with
           the issue fraction from the committed ncu summary); for a pair
           body chosen with --pair-variant, 10 flops per evaluated pair (12
           for the symmetric bodies) against the FP32 CUDA-core peak
cpu_baseline  the reference's OpenMP density algorithm (restated in C with
           its own linear window scans, all host cores) on a bounded sample

--impl reference times that CPU implementation alone (the reference arm).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "pair-kernel evals/s; MI/TE estimates/s batched+learned vs plain at |ΔH|≤1e-4 nats"
UNIT = "pair-kernel evals/s"
N_FRAMES, N_COORDS = 100_000, 64
WORKLOAD = "all-pairs MI, 64 coords x 100k frames, tanh(A z) AR(1) latent, Scott h"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-compare", action="store_true",
                    help="skip the batched+learned vs plain comparison")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the supplementary measurements of the other configurations")
    ap.add_argument("--pair-variant", default=None,
                    help="pair body per dimension, e.g. '4,4,4' (default: the library's)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the library's default tile shapes (no autotuner pass)")
    ap.add_argument("--cells-per-h3", type=int, default=0,
                    help="cells per bandwidth of 3-D strips (1 or 2; default: the library's)")
    ap.add_argument("--te-coords", type=int, default=0,
                    help="time only the transfer-entropy batch over the first N coordinates of "
                         "the 32 x 200k Langevin data (lags 1, 5, 10): the small case for ncu "
                         "captures of the 3-D kernel; prints a JSON line of its own")
    ap.add_argument("--xtc-frames", type=int, default=0,
                    help="time only the XTC trajectory load (1000 atoms x N frames): the small "
                         "case for ncu captures of the decode kernel; prints a JSON line of its "
                         "own")
    ap.add_argument("--xtc-atoms", type=int, default=1000,
                    help="atoms of the --xtc-frames trajectory (default 1000)")
    ap.add_argument("--coords-file", action="store_true",
                    help="time only the ASCII coordinate-file reader and device loader on the "
                         "64 x 100k MI matrix; prints a JSON line of its own")
    ap.add_argument("--coords", type=int, default=N_COORDS,
                    help="coordinates of the MI batch (64 = the benchmark workload; "
                         "smaller values give the small case used for ncu captures)")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *exc):
        if self.p is not None:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()

    def summary(self):
        self.f.flush()
        rows = []
        for ln in Path(self.f.name).read_text().splitlines():
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows),
                "sm_max_mhz": max(r[1] for r in rows), "reasons": reasons, "samples": len(rows)}


def fp32_peak_tflops(n_sms: int) -> tuple[float, str]:
    mhz = 2070.0
    try:
        mp = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
        mhz = float(mp.get("sm_max_mhz", mhz))
    except Exception:
        pass
    peak = n_sms * 128 * 2 * mhz * 1e6 / 1e12
    return peak, (f"nominal FP32 CUDA-core peak {n_sms} SMs x 128 FMA/clk x 2 x {mhz:.0f} MHz "
                  "(no measured FP32 figure in MEASURED_PEAKS.json)")


# Compulsory HBM bytes per 2-D point of the strip-moment group (one MI step,
# log-sum epilogue): the point (8 B) read by the strip-extent, moment-total,
# prefix-write and target kernels (4 x 8) and by the edge kernel as a source
# and as a target (2 x 8), the 128 B moment prefix row written once, the strip
# key (4 B), and the FP64 edge sum written by the edge kernel and read by the
# target kernel (2 x 8). The target kernel re-reads the rows at its range
# ends from L2 (measured: 34 B per target from DRAM in all).
MOMENT_BYTES_PER_POINT = 4 * 8 + 2 * 8 + 128 + 4 + 2 * 8
def profile_figure(name: str, key: str) -> float | None:
    """A figure `key = value` from a committed ncu summary under profiles/."""
    p = ROOT / "profiles" / name
    if not p.exists():
        return None
    for ln in p.read_text().splitlines():
        if ln.startswith(key):
            try:
                return float(ln.split("=", 1)[1].split()[0])
            except Exception:
                return None
    return None


def hbm_peak_gbs() -> tuple[float, str]:
    try:
        mp = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
        return float(mp["hbm_gbs"]), "measured copy bandwidth (MEASURED_PEAKS.json hbm_gbs)"
    except Exception:
        return 6800.0, "fallback 6.8 TB/s (no MEASURED_PEAKS.json)"


def moment_roofline(t_target: float, t_edge: float, t2: float, points_2d: int,
                    edge_pairs: float) -> dict:
    """Roofline of the 2-D strip-moment group of the MI step (edge kernel,
    strip extents, moment prefix sums, target kernel; CUDA events on the
    library stream): compulsory HBM bytes over the group's time, against the
    measured copy bandwidth, with the DRAM bytes ncu measured for the same
    kernels (small case, scaled by points). Beside it, each of the two largest
    kernels timed on its own: the target kernel k_m2_density (dominant;
    dependent L1/L2 loads of the binary searches and 128-bit moment rows) and
    the symmetric edge kernel (12 flops per candidate pair against the FP32
    peak), with their ncu issue and FMA-pipe fractions."""
    import torch
    peak, note = hbm_peak_gbs()
    achieved = MOMENT_BYTES_PER_POINT * points_2d / t2 / 1e9
    prof = "moments2d_mi64x100k_ncu.md"
    fpeak, fnote = fp32_peak_tflops(torch.cuda.get_device_properties(0).multi_processor_count)
    edge_tflops = 12.0 * edge_pairs / t_edge / 1e12
    per_pt = profile_figure(prof, "dram_bytes_per_point")
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak,
            "traffic": per_pt * points_2d if per_pt else None,
            "kernel": "2-D strip-moment group: k_m2_density, k_density_sym (edge strips), "
                      "k_m2_write, k_m2_totals, k_m2_ybounds, k_m2_chunks",
            "bytes_per_point": MOMENT_BYTES_PER_POINT, "points_2d": points_2d,
            "group_ms": t2 * 1e3, "peak_kind": note,
            "target_kernel": {"kernel": "k_m2_density", "ms": t_target * 1e3,
                              "share_of_group": t_target / t2,
                              "issue_frac_ncu": profile_figure(prof, "issue_frac"),
                              "dram_bytes_per_target_ncu":
                                  profile_figure(prof, "target_dram_bytes_per_target"),
                              "bound": "dependent L1/L2 loads (long-scoreboard stalls)"},
            "edge_kernel": {"kernel": "k_density_sym<2,32,4,4> (edge strips)",
                            "ms": t_edge * 1e3, "share_of_group": t_edge / t2,
                            "candidate_pairs": edge_pairs,
                            "achieved_tflops": edge_tflops, "peak_tflops": fpeak,
                            "frac": edge_tflops / fpeak,
                            "fma_pipe_frac_ncu": profile_figure(prof, "edge_fma_pipe_frac"),
                            "peak_kind": fnote}}


def roofline_3d(pairs: float, ms: float) -> dict:
    """The 3-D symmetric pair kernel against the FP32 CUDA-core peak: 14
    flops per evaluated unordered pair (its body), with the FMA-pipe busy
    fraction of the committed ncu summary."""
    import torch
    peak, note = fp32_peak_tflops(torch.cuda.get_device_properties(0).multi_processor_count)
    prof = "density3d_sym_te4_ncu.md"
    fpp = profile_figure(prof, "flops_per_pair") or 14.0
    achieved = fpp * pairs / (ms / 1e3) / 1e12
    return {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "kernel": "k_density_sym<3,16,5,4>", "flops_per_pair": fpp,
            "ordered_equivalent_tflops": 30.0 * pairs / (ms / 1e3) / 1e12,
            "fma_pipe_frac_ncu": profile_figure(prof, "fma_pipe_frac"), "peak_kind": note}


def ncu_traffic() -> float | None:
    """DRAM bytes per launch of the 2-D pair kernel from the committed ncu
    summary (profiles/), if one has been captured."""
    p = ROOT / "profiles" / "density2d_sym_mi8x100k_ncu.md"
    if not p.exists():
        return None
    for ln in p.read_text().splitlines():
        if ln.startswith("dram_bytes_per_launch"):
            try:
                return float(ln.split("=", 1)[1].split()[0])
            except Exception:
                return None
    return None


def cpu_port_sample(x: np.ndarray, h: np.ndarray, pairs, support):
    """Time the reference OpenMP density algorithm (restated, with its linear
    window scans) on the given instances; returns (pairs/s, seconds, n)."""
    from oracle import oracle as O
    t0 = time.perf_counter()
    for inst in pairs:
        O.density_ref_f32(O.repack(x, list(inst)), [h[c] for c in inst], linear_scan=True)
    dt = time.perf_counter() - t0
    return support / dt, dt


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else platform)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.strip().startswith("Model name:"):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for ln in Path("/proc/cpuinfo").read_text().splitlines():
            if ln.startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.processor() or platform.machine()


def timed_port(fn):
    """(result, seconds) of one call of the reference algorithm restated."""
    t0 = time.perf_counter()
    r = fn()
    return r, time.perf_counter() - t0


def learned_heldout(ctx, n_held=256, n_fp64=16):
    """Config 5 held out: 256 generated mixtures (d 1..3, N log-uniform in
    [5k, 200k], the training generator with another seed), bandwidths by the
    full AMISE search, by the network's warm start and by the constant-offset
    warm start (no network); search passes, fallbacks and bandwidth/entropy
    differences per arm, and |dH| against the FP64 oracle on a seeded sample
    of n_fp64 mixtures of at most 50k frames (entropy at each warm start's
    bandwidths vs the FP64 entropy at the full search's)."""
    from entropical_gb300 import learned
    from oracle import oracle as O
    net = learned.BandwidthMLP.load(ctx)
    held = learned.generate(n_held, seed=777)
    t0 = time.perf_counter()
    ev = learned.evaluate(ctx, net, held)
    t_eval = time.perf_counter() - t0
    small = [q for q, x in enumerate(held) if x.shape[1] <= 50_000]
    rng = np.random.default_rng(1)
    pick = sorted(rng.choice(small, min(n_fp64, len(small)), replace=False).tolist())
    err = 0.0
    t0 = time.perf_counter()
    for q in pick:
        x = held[q]
        err = max(err, abs(ev["H_full"][q] - O.entropy_fp64(x, ev["h_full"][q, :x.shape[0]])))
    out = {k: v for k, v in ev.items() if k not in ("h_full", "H_full")}
    out.update({"workload": f"{n_held} held-out mixtures, d 1-3, N 5k-200k (seed 777)",
                "eval_s": t_eval,
                "max_abs_dH_vs_fp64_oracle": err, "fp64_oracle_mixtures": len(pick),
                "fp64_oracle_s": time.perf_counter() - t0,
                "note": "network and constant arms identical: the reference's AMISE objective "
                        "falls monotonically in h, so every label is the same ratio "
                        f"{learned.CONSTANT_RATIO}"})
    return out


def compare_plain(ctx, pctx, x, ptr, log_fp64_pairs=2):
    """Bandwidths by the AMISE search and then all-pairs MI, two ways:
    plain  -- the single-instance entry points called the way the reference
              calls them: per column 16 epa_convolution calls driven by the
              AmiseMin bracket logic (hestimate.cpp:55-104), then mi.cpp's loop
              (per pair the 1-D marginal again and the 2-D joint, mi.cpp:37-59);
    batched+learned -- ent_hestimate_learned (features, network, warm search
              for all columns at once) and one ent_mi_all_pairs batch.
    The plain side runs on its own context pctx with the library defaults
    (the body each single call is fastest with), the batched side on ctx.
    Returns a dict of times, convolution counts and MI differences."""
    from entropical_gb300 import learned
    from entropical_gb300.densities import HEST_THUMB
    from entropical_gb300.estimators import hestimate_amise_plain
    M, N = x.shape
    torch_sync = __import__("torch").cuda.synchronize
    torch_sync()
    t0 = time.perf_counter()
    h0, _ = pctx.hestimate(x, HEST_THUMB)
    h_plain, calls = np.zeros(M, np.float32), 0
    for j in range(M):
        hj, c = hestimate_amise_plain(pctx, x[j], float(h0[j]))
        h_plain[j], calls = hj, calls + c
    t_hest_plain = time.perf_counter() - t0
    t0 = time.perf_counter()
    mi_plain = np.zeros((M, M))
    for i in range(M):
        Hi = -np.mean(np.log(pctx.combined_densities(x, None, [i], [h_plain[i]])))
        for j in range(i + 1, M):
            Hj = -np.mean(np.log(pctx.combined_densities(x, None, [j], [h_plain[j]])))
            Hij = -np.mean(np.log(pctx.combined_densities(x, None, [i, j],
                                                         [h_plain[i], h_plain[j]])))
            mi_plain[i, j] = mi_plain[j, i] = Hi + Hj - Hij
    t_mi_plain = time.perf_counter() - t0
    net = learned.BandwidthMLP.load(ctx)
    items = [(ptr + 4 * N * j, 1, N) for j in range(M)]
    learned.hestimate_learned(ctx, net, items, skip_levels=6, device=True)  # warm-up
    torch_sync()
    t0 = time.perf_counter()
    hl, st = learned.hestimate_learned(ctx, net, items, skip_levels=6, device=True)
    t_hest_l = time.perf_counter() - t0
    t0 = time.perf_counter()
    mi_b, _ = ctx.mi_all_pairs_device(ptr, N, M, hl[:, 0])
    t_mi_b = time.perf_counter() - t0
    iu = np.triu_indices(M, 1)
    out = {
        "workload": "AMISE bandwidths for 64 columns, then all-pairs MI (64 x 100k)",
        "plain_s": t_hest_plain + t_mi_plain, "plain_hestimate_s": t_hest_plain,
        "plain_mi_s": t_mi_plain, "plain_density_calls": M + 2 * len(iu[0]),
        "plain_conv_calls": calls,
        "batched_learned_s": t_hest_l + t_mi_b, "learned_hestimate_s": t_hest_l,
        "batched_mi_s": t_mi_b,
        "learned_conv_evals": int(sum(s[0]["conv_evals"] for s in st)),
        "learned_fallbacks": int(sum(1 - s[0]["warm_converged"] for s in st)),
        "bandwidths_identical": bool(np.array_equal(hl[:, 0], h_plain)),
        "max_abs_dI_batched_vs_plain": float(np.max(np.abs(mi_b - mi_plain)[iu])),
    }
    out["speedup"] = out["plain_s"] / out["batched_learned_s"]
    try:
        from oracle import oracle as O
        errs = []
        for (i, j) in [(0, 1), (5, 40)][:log_fp64_pairs]:
            ref = O.mi_fp64(x[i], x[j], float(h_plain[i]), float(h_plain[j]))
            errs.append(abs(mi_b[i, j] - ref))
        out["max_abs_dI_vs_fp64_oracle"] = max(errs)
        out["fp64_oracle_pairs"] = log_fp64_pairs
        # CPU baseline of the bandwidth search: the reference's AMISE
        # convolution (O(N^2), all host threads) on the sorted first 20,000
        # frames of two columns, extrapolated to 16 convolutions per column,
        # N = 100k (x (100k / 20k)^2) and 64 columns
        ts = []
        for c in (0, 1):
            col = np.sort(x[c][:20_000])
            _, t = timed_port(lambda: O.epa_conv_ref(col, float(h_plain[c])))
            ts.append(t)
        per_col = statistics.mean(ts) * 16 * (N / 20_000) ** 2
        out["cpu_baseline_amise"] = {"sample_s": sum(ts), "cores": os.cpu_count(),
                                     "sample": "one convolution on 20k sorted frames of 2 columns",
                                     "extrapolated_per_column_s": per_col,
                                     "extrapolated_64_columns_s": 64 * per_col, "kind": "port"}
    except Exception as exc:
        out["fp64_oracle_error"] = str(exc)[:200]
    return out


def compare_plain_te(ctx, pctx, n_coords=32, taus=(1, 5, 10)):
    """Transfer entropy of all ordered pairs over the first n_coords of the
    coupled-Langevin data (200k frames, 3 lags), bandwidths by the AMISE
    search, two ways: plain -- per column 16 epa_convolution calls driven by
    the AmiseMin bracket logic, then one density call per density the TE
    estimates need (1-D, 2-D lagged, 2-D joint, 3-D; transs.cpp:39-115
    structure); batched+learned -- ent_hestimate_learned for all columns and
    one ent_te_all_pairs batch for all pairs and lags. The plain side runs on
    its own default context pctx."""
    from entropical_gb300 import learned, workloads
    from entropical_gb300.densities import HEST_THUMB
    from entropical_gb300.estimators import hestimate_amise_plain
    xt, _ = workloads.langevin(32, 200_000, seed=11)
    x = np.ascontiguousarray(xt[:n_coords])
    M, N = x.shape
    sync = __import__("torch").cuda.synchronize
    sync()
    t0 = time.perf_counter()
    h0, _ = pctx.hestimate(x, HEST_THUMB)
    hp = np.array([hestimate_amise_plain(pctx, x[j], float(h0[j]))[0] for j in range(M)],
                  np.float32)
    calls, te_plain = 0, np.zeros((len(taus), M, M))
    for q, tau in enumerate(taus):
        n = N - tau
        xn = np.ascontiguousarray(x[:, :n])  # the n samples t of y_i and x_j
        H1 = [-np.mean(np.log(pctx.combined_densities(xn, None, [i], [hp[i]])))
              for i in range(M)]
        Hl = [-np.mean(np.log(pctx.combined_densities(x, None, [i, i], [hp[i], hp[i]], [tau, 0])))
              for i in range(M)]
        calls += 2 * M
        for i in range(M):
            for j in range(M):
                if i == j:
                    continue
                H2 = -np.mean(np.log(pctx.combined_densities(xn, None, [i, j],
                                                            [hp[i], hp[j]])))
                H3 = -np.mean(np.log(pctx.combined_densities(
                    x, None, [i, i, j], [hp[i], hp[i], hp[j]], [tau, 0, 0])))
                calls += 2
                te_plain[q, i, j] = H2 + Hl[i] - H3 - H1[i]
    t_plain = time.perf_counter() - t0
    net = learned.BandwidthMLP.load(ctx)
    learned.hestimate_learned(ctx, net, list(x), skip_levels=6)  # warm-up
    ctx.te_all_pairs(x, hp, list(taus))
    sync()
    t0 = time.perf_counter()
    hl, st = learned.hestimate_learned(ctx, net, list(x), skip_levels=6)
    t_h = time.perf_counter() - t0
    te_b = ctx.te_all_pairs(x, hl[:, 0], list(taus))
    t_b = time.perf_counter() - t0
    cs = ctx.last_stats()
    off = ~np.eye(M, dtype=bool)
    return {"workload": f"AMISE bandwidths for {M} columns, then TE of all {M * (M - 1)} ordered "
                        f"pairs at lags {list(taus)} ({M} x {N} Langevin)",
            "plain_s": t_plain, "plain_density_calls": calls, "batched_learned_s": t_b,
            "learned_hestimate_s": t_h, "batched_te_device_ms": cs.total_ms,
            "batched_te_pair_kernel_ms_by_dim": list(cs.pair_kernel_ms_by_dim),
            "h_over_scott_median": float(np.median(hl[:, 0] / workloads.scott_bandwidth(x, 3))),
            "speedup": t_plain / t_b, "te_estimates": int(len(taus) * M * (M - 1)),
            "bandwidths_identical": bool(np.array_equal(hl[:, 0], hp)),
            "max_abs_dTE_batched_vs_plain": float(np.max(np.abs(te_b - te_plain)[:, off])),
            "learned_fallbacks": int(sum(1 - s[0]["warm_converged"] for s in st))}


def other_configs(ctx):
    """The other configurations, measured once (device time of one call each):
    config 1 (1-D GMM density), config 3 (TE, all ordered pairs, 3 lags) and
    config 4 (512 uneven instances: one batch vs sequential plain calls)."""
    from entropical_gb300 import workloads
    out = {}
    x1 = workloads.gmm_1d(20_000, seed=42)[None]
    ctx.combined_densities(x1, None, [0], [0.1])
    ctx.combined_densities(x1, None, [0], [0.1])
    st = ctx.last_stats()
    sup = float(ctx.support_counts(x1, None, [0], [0.1]).sum())
    p1 = ctx.combined_densities(x1, None, [0], [0.1])
    from oracle import oracle as O
    f1 = O.density_fp64(x1, [0.1])
    _, t_cpu1 = timed_port(lambda: O.density_ref_f32(x1, [0.1], linear_scan=True))
    # 1-D range sums: the point read by the prefix, target and finish kernels
    # (3 x 4 B), its 32 B prefix row written and read (2 x 32 B), the sort
    # (4 passes x 16 B) and the FP64 output (8 B), over the pair-kernel time
    peak_hbm, _ = hbm_peak_gbs()
    b1 = (3 * 4 + 2 * 32 + 4 * 16 + 8) * x1.shape[1]
    out["gmm1d_20k"] = {"ms": st.total_ms, "support_pairs": sup,
                        "pairs_per_s": sup / (st.total_ms / 1e3),
                        "roofline": {"bound": "hbm", "bytes": b1, "achieved_gbs":
                                     b1 / (st.total_ms / 1e3) / 1e9,
                                     "frac": b1 / (st.total_ms / 1e3) / 1e9 / peak_hbm,
                                     "note": "20k points stay in L2; the call is bound by its "
                                             "launch sequence (about 20 kernels), not by HBM"},
                        "max_rel_err_density_vs_fp64": float(np.max(np.abs(p1 - f1) / f1)),
                        "max_abs_err_vs_fp64": abs(float(-np.mean(np.log(p1)))
                                                   - float(-np.mean(np.log(f1)))),
                        "cpu_baseline": {"s": t_cpu1, "pairs_per_s": sup / t_cpu1,
                                         "sample": "the full configuration", "kind": "port"}}
    xt, _ = workloads.langevin(32, 200_000, seed=11)
    ht = workloads.scott_bandwidth(xt, 3)
    taus = [1, 5, 10]
    # device time of one call: the better of two
    te = ctx.te_all_pairs(xt, ht, taus)
    st = ctx.last_stats()
    te = ctx.te_all_pairs(xt, ht, taus)
    if ctx.last_stats().total_ms < st.total_ms:
        st = ctx.last_stats()
    cnt = ctx.te_all_pairs(xt, ht, taus, counts=True)
    sup3 = float(cnt.sum() - sum(np.trace(c) for c in cnt))
    # FP64 error on four sampled (pair, lag) entries; te[q, i, j] = TE_{j->i}
    rng = np.random.default_rng(3)
    te_err, t0 = 0.0, time.perf_counter()
    for _ in range(4):
        q = int(rng.integers(3))
        i, j = (int(v) for v in rng.choice(32, 2, replace=False))
        ref = O.te_fp64(xt[j], xt[i], taus[q], float(ht[j]), float(ht[i]))
        te_err = max(te_err, abs(te[q, i, j] - ref))
    t_fp64 = time.perf_counter() - t0
    # CPU baseline: the 3-D density of one (pair, lag), extrapolated to the
    # batch by in-support pairs
    sel3 = O.repack(xt, [5, 5, 17], [5, 0, 0])
    _, t_cpu3 = timed_port(lambda: O.density_ref_f32(sel3, [ht[5], ht[5], ht[17]],
                                                     linear_scan=True))
    sup_s3 = float(O.support_count_fp64(sel3, [ht[5], ht[5], ht[17]]))
    out["te_32x200k_3lags"] = {
        "ms": st.total_ms, "densities": st.instances, "te_estimates": 3 * 32 * 31,
        "te_estimates_per_s": 3 * 32 * 31 / (st.total_ms / 1e3),
        "pair_kernel_ms_by_dim": list(st.pair_kernel_ms_by_dim),
        "support_pairs_3d": sup3, "candidate_pairs_3d": st.candidate_pairs_by_dim[2],
        "h2d_bytes": int(xt.nbytes),
        "max_abs_err_vs_fp64": te_err, "fp64_oracle_entries": 4, "fp64_oracle_s": t_fp64,
        "roofline_3d": roofline_3d(st.candidate_pairs_by_dim[2], st.pair_kernel_ms_by_dim[2]),
        "moment_target_ms": st.moment_target_ms, "moment_edge_ms": st.moment_edge_ms,
        "cpu_baseline": {"s": t_cpu3, "pairs_per_s": sup_s3 / t_cpu3,
                         "sample": "3-D density (x5[t+5], x5[t], x17[t]) at 200k frames",
                         "extrapolated_3d_s": sup3 / (sup_s3 / t_cpu3), "kind": "port"}}
    ub = workloads.uneven_batch(512, seed=5)
    # tile/cell shapes per dimension picked by the autotuner on this batch
    from entropical_gb300 import Context, autotune
    uctx = Context(-1)
    utuned = {f"d{d}": {k: v for k, v in autotune.tune(uctx, lambda: uctx.entropy_batch(ub), d=d,
                                                       n=100_000, repeats=1, save=False).items()
                        if k != "all"} for d in (1, 2, 3)}
    # first call grows the context's workspace, the next may coalesce it:
    # the best of three calls after that
    H = uctx.entropy_batch(ub)
    st = None
    for _ in range(3):
        H = uctx.entropy_batch(ub)
        if st is None or uctx.last_stats().total_ms < st.total_ms:
            st = uctx.last_stats()
    uctx.close()
    supu = float(ctx.entropy_batch(ub, counts=True).sum())
    t0 = time.perf_counter()
    for xq, hq in ub:
        ctx.combined_densities(xq, None, list(range(xq.shape[0])), hq)
    seq = time.perf_counter() - t0
    # FP64 entropy of the smallest and the largest instance of each dimension
    by_d = {d: sorted((q for q, (xq, _) in enumerate(ub) if xq.shape[0] == d),
                      key=lambda q: ub[q][0].shape[1]) for d in (1, 2, 3)}
    u_err, t0 = 0.0, time.perf_counter()
    for d in (1, 2, 3):
        for q in (by_d[d][0], by_d[d][-1]):
            u_err = max(u_err, abs(H[q] - O.entropy_fp64(*ub[q])))
    t_fp64u = time.perf_counter() - t0
    # CPU baseline: a stratified sample (per dimension the instances at the
    # 10th, 50th and 90th size percentile), extrapolated by in-support pairs
    samp = [by_d[d][int(f * (len(by_d[d]) - 1))] for d in (1, 2, 3) for f in (0.1, 0.5, 0.9)]
    t0 = time.perf_counter()
    for q in samp:
        O.density_ref_f32(*ub[q], linear_scan=True)
    t_cpuu = time.perf_counter() - t0
    sup_su = float(sum(O.support_count_fp64(*ub[q]) for q in samp))
    import torch
    fpeak, _ = fp32_peak_tflops(torch.cuda.get_device_properties(0).multi_processor_count)
    # flops per candidate pair of the chosen bodies: symmetric 12 (2-D) / 14
    # (3-D) per unordered pair, ordered 5 d; range sums and moments have none
    fl_u = {}
    for d in (1, 2, 3):
        v = utuned[f"d{d}"]["pair_variant"]
        f = {1: 12.0, 2: 12.0, 3: 14.0}[d] if v in (4, 5) else (5.0 * d if v <= 3 else 0.0)
        ms_d = st.pair_kernel_ms_by_dim[d - 1]
        tf = f * st.candidate_pairs_by_dim[d - 1] / (ms_d / 1e3) / 1e12 if f and ms_d else None
        fl_u[f"d{d}"] = {"pair_variant": v, "flops_per_pair": f, "tflops": tf,
                         "frac": tf / fpeak if tf else None}
    out["uneven_512"] = {"batched_ms": st.total_ms, "sequential_plain_s": seq, "autotuned": utuned,
                         "roofline_by_dim": fl_u,
                         "max_abs_err_vs_fp64": u_err, "fp64_oracle_instances": 6,
                         "fp64_oracle_s": t_fp64u,
                         "cpu_baseline": {"s": t_cpuu, "pairs_per_s": sup_su / t_cpuu,
                                          "sample": "9 instances: per dimension the 10th, 50th "
                                                    "and 90th size percentile",
                                          "extrapolated_s": supu / (sup_su / t_cpuu),
                                          "kind": "port"},
                         "pair_kernel_ms_by_dim": list(st.pair_kernel_ms_by_dim),
                         "candidate_pairs_by_dim": list(st.candidate_pairs_by_dim),
                         "speedup": seq / (st.total_ms / 1e3), "support_pairs": supu,
                         "pairs_per_s": supu / (st.total_ms / 1e3),
                         "points": int(sum(xq.shape[1] for xq, _ in ub))}
    # the reference's own estimator formulas, one device batch each
    from entropical_gb300.densities import REF_MI, REF_TRANSS
    xm = workloads.mi_coords(100_000, 64, seed=2024)
    hm = workloads.scott_bandwidth(xm, 2)
    ref = {}
    for name, xx, hh, kind, tau in (("mi_64x100k", xm, hm, REF_MI, 0),
                                    ("transs_32x200k_tau5", xt, ht, REF_TRANSS, 5)):
        ctx.reference_estimator(xx, hh, kind, tau)
        st = ctx.last_stats()
        ref[name] = {"ms": st.total_ms, "densities": st.instances,
                     "pair_kernel_ms_by_dim": list(st.pair_kernel_ms_by_dim)}
    d3 = ctx.dens_all(xm[:16], hm[:16], 3)
    st = ctx.last_stats()
    ref["dens_D3_16x100k"] = {"ms": st.total_ms, "densities": int(d3.shape[0]),
                              "d2h_bytes": int(d3.nbytes)}
    out["reference_formulas"] = ref
    out["coords_file_64x100k"] = coords_file_config(ctx, xm)
    out["xtc_1000atoms_50k"] = xtc_config(ctx)
    return out


def coords_file_config(ctx, xm: np.ndarray, reps: int = 3) -> dict:
    """The reference's ASCII coordinate format (Tools::IO::read_coords,
    tools.hxx:153-235) for the MI matrix, written with 9 significant digits
    (which give every float back exactly): the parallel host parse (shape,
    then values, as the reference's two passes), and the device loader with
    pinned, overlapped copies. Best of `reps` calls each, the file in the
    page cache."""
    import tempfile
    import torch
    from entropical_gb300 import read_coords
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "coords.txt")
        np.savetxt(path, xm.T, fmt="%.9g")
        size = os.path.getsize(path)
        t_host, t_dev = [], []
        for _ in range(reps):
            t0 = time.perf_counter()
            host = read_coords(path)
            t_host.append(time.perf_counter() - t0)
        dev = torch.empty(host.shape, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        for _ in range(reps):
            t0 = time.perf_counter()
            ctx.load_coords_device(path, dev.data_ptr())
            torch.cuda.synchronize()
            t_dev.append(time.perf_counter() - t0)
        same = bool(torch.equal(dev.cpu(), torch.from_numpy(host)))
        exact = bool(np.array_equal(host, xm.astype(np.float32)))
    t_h, t_d = min(t_host), min(t_dev)
    return {"bytes": size, "values": int(xm.size), "read_s": t_h,
            "read_MB_per_s": size / t_h / 1e6, "load_device_s": t_d,
            "load_device_MB_per_s": size / t_d / 1e6, "reps": reps,
            "device_equals_host": same, "host_equals_values_written": exact,
            "threads": os.cpu_count()}


def xtc_trajectory(n_atoms: int, n_frames: int, seed: int = 21) -> np.ndarray:
    """Synthetic MD-like frames (n_frames, 3 n_atoms): a chain of a quarter of
    the atoms with 0.15 nm steps drifting as a whole, and three-atom water
    molecules for the rest in a 5 nm box, every atom jittered by 0.03 nm per
    frame."""
    rng = np.random.default_rng(seed)
    n_chain = n_atoms // 4
    n_mol = (n_atoms - n_chain) // 3
    chain = np.cumsum(rng.normal(0, 0.15, (n_chain, 3)), 0) + 2.5
    o = rng.uniform(0, 5.0, (n_mol, 1, 3))
    water = np.concatenate([o, o + rng.normal(0, 0.06, (n_mol, 2, 3))], 1).reshape(-1, 3)
    base = np.concatenate([chain, water]).astype(np.float32)
    drift = np.cumsum(rng.normal(0, 0.002, (n_frames, 1, 3)), 0).astype(np.float32)
    rows = np.empty((n_frames, 3 * len(base)), np.float32)
    for f0 in range(0, n_frames, 5000):
        f1 = min(n_frames, f0 + 5000)
        jit = rng.normal(0, 0.03, (f1 - f0, len(base), 3)).astype(np.float32)
        fr = base[None] + jit
        fr[:, :n_chain] += drift[f0:f1]
        rows[f0:f1] = fr.reshape(f1 - f0, -1)
    return rows


def xtc_config(ctx, n_atoms: int = 1000, n_frames: int = 50_000):
    """XTC trajectory input (CoordsFile::XtcHandler, coords_file.cpp:70-126):
    write a synthetic trajectory with the library's writer, then load it into
    a column-major device matrix (ent_load_xtc_device: host index, pinned
    copies of the compressed file, a walk per frame, one decoding thread per
    64-atom segment). Times the
    load (best of 3, wall, from the page cache) and the decode kernel, checks
    sampled frames against the oracle's reader bit for bit, and times the
    oracle's serial reader (the reference reads frame by frame with read_xtc)
    on a sample."""
    import tempfile
    import torch
    from entropical_gb300 import write_xtc, xtc_file_shape
    from oracle import oracle as O
    rows = xtc_trajectory(n_atoms, n_frames)
    out = {"workload": f"{n_atoms} atoms x {n_frames} frames ({3 * n_atoms} coordinates), "
                       "chain + water, precision 1000"}
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "traj.xtc")
        t0 = time.perf_counter()
        write_xtc(path, rows, primary="R")
        out["write_s"] = time.perf_counter() - t0
        size = os.path.getsize(path)
        dev = torch.empty((3 * n_atoms, n_frames), dtype=torch.float32, device="cuda")
        ctx.load_xtc_device(path, dev.data_ptr())  # warm-up (and page cache)
        walls, kern = [], []
        for _ in range(3):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ctx.load_xtc_device(path, dev.data_ptr())
            torch.cuda.synchronize()
            walls.append(time.perf_counter() - t0)
            kern.append(ctx.last_stats().pair_kernel_ms)
        wall, k_ms = min(walls), float(np.median(kern))
        t0 = time.perf_counter()
        xtc_file_shape(path)
        t_index = time.perf_counter() - t0
        sample = min(2000, n_frames)
        got = dev[:, :sample].cpu().numpy()
        t0 = time.perf_counter()
        want = O.read_xtc(path, 0, sample)
        t_cpu = time.perf_counter() - t0
        exact = bool(np.array_equal(got.T.view(np.uint32), want.view(np.uint32)))
        last = dev[:, -1].cpu().numpy()
        exact = exact and bool(np.array_equal(last.view(np.uint32),
                                              O.read_xtc(path, n_frames - 1)[0].view(np.uint32)))
    out_bytes = 4 * 3 * n_atoms * n_frames
    peak, peak_kind = hbm_peak_gbs()
    out.update({
        "file_bytes": size, "bytes_per_coordinate": size / (3 * n_atoms * n_frames),
        "load_device_s": wall, "load_device_MB_per_s": size / wall / 1e6,
        "coordinates_per_s": 3 * n_atoms * n_frames / wall,
        "decode_kernel_ms": k_ms, "index_s": t_index,
        "decode_roofline": {"bound": "latency (a dependent walk per frame over its atom "
                                     "groups, then one thread per 64-atom segment)",
                            "algorithmic_bytes": size + out_bytes,
                            "achieved_gbs": (size + out_bytes) / (k_ms / 1e3) / 1e9,
                            "peak_gbs": peak, "frac": (size + out_bytes) / (k_ms / 1e3) / 1e9 / peak,
                            "peak_kind": peak_kind},
        "bit_exact_vs_oracle": exact, "oracle_frames_checked": sample + 1,
        "cpu_baseline": {"s": t_cpu, "frames": sample, "cores": 1, "kind": "port",
                         "sample": f"frames 0-{sample - 1} decoded serially by the oracle's "
                                   "read_xtc restatement",
                         "extrapolated_s": t_cpu * n_frames / sample},
    })
    return out


def reference_arm(args, x, h):
    """The reference's OpenMP algorithm (restated in C, linear window scans
    kept, all host threads) on the same MI job as the GPU arm. Each step
    times a seeded sample of it -- one 1-D marginal and one 2-D joint, a
    different pair every step -- and extrapolates to the whole job (64
    marginals, 2,016 joints) from the sample's in-support pairs per second
    per dimension; value = the job's in-support pairs / extrapolated time."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    M = x.shape[0]
    iu = np.triu_indices(M, 1)
    rng = np.random.default_rng(2024)
    order = rng.permutation(len(iu[0]))
    # in-support pairs of the whole job, by dimension (FP64 counts, untimed)
    sup1 = [O.support_count_fp64(x[c][None], [h[c]]) for c in range(M)]
    job1 = float(sum(sup1))
    rates, times = [], []
    for s in range(args.warmup + args.steps):
        q = int(order[s % len(order)])
        i, j = int(iu[0][q]), int(iu[1][q])
        sel = O.repack(x, [i, j])
        sup2 = O.support_count_fp64(sel, [h[i], h[j]])
        r1, t1 = cpu_port_sample(x, h, [(i,)], sup1[i])
        r2, t2 = cpu_port_sample(x, h, [(i, j)], sup2)
        # the job's 2-D pairs: this pair's rate times the 2,016 joints
        job2 = float(sup2) * len(iu[0])
        job_s = job1 / r1 + job2 / r2
        if s >= args.warmup:
            rates.append((job1 + job2) / job_s)
            times.append(t1 + t2)
    v = statistics.mean(rates)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD,
                   "step": "a seeded sample of the same job: one 1-D marginal and one 2-D joint "
                           "(another pair each step), extrapolated to 64 marginals + 2,016 "
                           "joints by in-support pairs",
                   "parallelism": f"OpenMP {cores} host threads", "same_job": True},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "cpu_model": cpu_model(),
                         "sample": "per step one 1-D marginal + one 2-D joint at N=100k, reference "
                                   "OpenMP algorithm restated in C (linear window scans kept), "
                                   "extrapolated to the 2,080-density MI job"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def te_only(args):
    """Transfer entropy of all ordered pairs of the first --te-coords
    Langevin coordinates (200k frames, lags 1, 5, 10), device time per call."""
    import torch
    from entropical_gb300 import Context, workloads
    xt, _ = workloads.langevin(32, 200_000, seed=11)
    x = np.ascontiguousarray(xt[:args.te_coords])
    h = workloads.scott_bandwidth(xt, 3)[:args.te_coords]
    ctx = Context(0)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(args.warmup):
        ctx.te_all_pairs(x, h, [1, 5, 10])
    ms, by_dim = [], []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        ctx.te_all_pairs(x, h, [1, 5, 10])
        st = ctx.last_stats()
        ms.append(st.total_ms)
        by_dim.append(list(st.pair_kernel_ms_by_dim))
    print(json.dumps({"workload": f"TE, {x.shape[0]} coords x 200k, lags 1, 5, 10",
                      "ms": statistics.mean(ms), "pair_kernel_ms_by_dim": by_dim[-1],
                      "candidate_pairs_by_dim": list(ctx.last_stats().candidate_pairs_by_dim)}),
          flush=True)


def main():
    args = parse()
    if args.te_coords:
        return te_only(args)
    if args.xtc_frames:
        from entropical_gb300 import Context
        print(json.dumps(xtc_config(Context(), n_atoms=args.xtc_atoms, n_frames=args.xtc_frames)))
        return None
    if args.coords_file:
        from entropical_gb300 import Context, workloads
        xm = workloads.mi_coords(N_FRAMES, N_COORDS, seed=2024)
        print(json.dumps(coords_file_config(Context(), xm)))
        return None
    ws, rank, local = dist_env()
    from entropical_gb300 import workloads
    # weak scaling over independent problems: rank r computes the benchmark
    # workload on its own data (seed + r); rank 0 alone is the 1-GPU case
    x = workloads.mi_coords(N_FRAMES, N_COORDS, seed=2024 + rank)[: args.coords]
    x = np.ascontiguousarray(x)
    h = workloads.scott_bandwidth(x, 2)
    M = x.shape[0]
    if args.impl == "reference":
        return reference_arm(args, x, h)

    import torch
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist_mod
        dist_mod.init_process_group("nccl")
        dist = dist_mod
    from entropical_gb300 import Context

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    ctx = Context(local)
    if args.pair_variant:
        ctx.set_tuning(pair_variant=[int(v) for v in args.pair_variant.split(",")])
    if args.cells_per_h3:
        ctx.set_tuning(cells_per_h3=args.cells_per_h3)
    n_sms = torch.cuda.get_device_properties(local).multi_processor_count
    dx = torch.from_numpy(x).cuda(local)
    ptr = dx.data_ptr()
    iu = np.triu_indices(M, 1)
    tuned = None
    if not (args.no_autotune or args.pair_variant or args.cells_per_h3):
        # tile/cell shapes picked by the autotuner on a sample of this batch
        # (the first 16 coordinates: 120 2-D and 16 1-D densities), untimed
        from entropical_gb300 import autotune
        ms = min(M, 16)
        run = lambda: ctx.mi_all_pairs_device(ptr, N_FRAMES, ms, h[:ms])  # noqa: E731
        tuned = {f"d{d}": {k: v for k, v in autotune.tune(ctx, run, d=d, n=N_FRAMES,
                                                           save=False).items() if k != "all"}
                 for d in (2, 1)}
    var2 = ctx.tuning()["pair_variant_by_dim"][1]

    # work units of the step: in-support (target, source) pairs (untimed)
    cnt, c1 = ctx.mi_all_pairs_device(ptr, N_FRAMES, M, h, counts=True)
    support_2d = float(cnt[iu].sum())
    support_1d = float(c1.sum())
    support = support_2d + support_1d

    for _ in range(args.warmup):
        mi, hx = ctx.mi_all_pairs_device(ptr, N_FRAMES, M, h)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    step_ms, k2_ms, k2_pairs, k1_ms, launches = [], [], [], [], 0
    km_ms, ke_ms = [], []
    barrier()
    wall0 = time.perf_counter()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()  # L2 flush between steps (256 MB > 129 MB L2)
            torch.cuda.synchronize()
            mi, hx = ctx.mi_all_pairs_device(ptr, N_FRAMES, M, h)
            st = ctx.last_stats()
            step_ms.append(st.total_ms)
            k2_ms.append(st.pair_kernel_ms_by_dim[1])
            k1_ms.append(st.pair_kernel_ms_by_dim[0])
            k2_pairs.append(st.candidate_pairs_by_dim[1])
            km_ms.append(st.moment_target_ms)
            ke_ms.append(st.moment_edge_ms)
            launches += st.kernel_launches
    barrier()
    wall = time.perf_counter() - wall0
    from entropical_gb300.replicas import aggregate
    units, ms = aggregate(support, statistics.mean(step_ms), dist, device=f"cuda:{local}")
    value = units / (ms / 1e3)

    # end to end through the host-buffer call (pinned host input)
    xp = torch.from_numpy(x).pin_memory()
    xnp = xp.numpy()
    e2e_ms = []
    for s in range(args.warmup + args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        mi_e, hx_e = ctx.mi_all_pairs(xnp, h)
        w = (time.perf_counter() - t0) * 1e3
        if s >= args.warmup:
            e2e_ms.append(max(w, ctx.last_stats().total_ms))
    e2e = statistics.mean(e2e_ms)
    assert np.allclose(mi_e, mi, rtol=0, atol=1e-9)
    # whole job, as value: the work of every rank over the slowest rank's time
    units_e2e, e2e = aggregate(support, e2e, dist, device=f"cuda:{local}")

    if rank != 0:
        return
    t2 = statistics.mean(k2_ms) / 1e3
    if var2 == 7:
        roofline = moment_roofline(statistics.mean(km_ms) / 1e3, statistics.mean(ke_ms) / 1e3,
                                   t2, M * (M - 1) // 2 * N_FRAMES, statistics.mean(k2_pairs))
    else:
        peak, peak_note = fp32_peak_tflops(n_sms)
        # symmetric bodies (4, 5) evaluate each unordered pair once and add it
        # to both points: 12 flops (6 FMA-pipe cycles) per evaluated pair
        fpp = 12 if var2 in (4, 5) else 10
        achieved = fpp * statistics.mean(k2_pairs) / t2 / 1e12
        roofline = {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                    "frac": achieved / peak, "traffic": ncu_traffic(),
                    "kernel": (f"k_density_sym<2,{32 if var2 == 4 else 16}> (2-D symmetric "
                               "pair kernel)" if var2 in (4, 5) else
                               f"k_density<2,16,{var2}> (2-D pair kernel)"),
                    "flops_per_pair": fpp, "peak_kind": peak_note}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD if M == N_COORDS else f"{WORKLOAD} (first {M} coords)",
                   "n_frames": N_FRAMES, "n_coords": M,
                   "densities_per_step": M + len(iu[0]), "l2": "flushed (256 MB write) "
                   "between steps", "parallelism": (f"{ws} independent problems, one per GPU (no collective on the "
                                   "data path)") if ws > 1 else "single GPU"},
        "mi_estimates_per_s": len(iu[0]) * ws / (ms / 1e3),
        "value_note": ("in-support (target, source) pairs of the step per second, counted once "
                       "per run by the ordered pair kernel; the default 1-D range sums and 2-D "
                       "strip moments sum most of them exactly without visiting each pair, so "
                       "the rate can exceed what the FP32 peak allows for pair-by-pair kernels"
                       if var2 == 7 else "in-support (target, source) pairs of the step per "
                       "second, counted once per run by the ordered pair kernel"),
        "support_pairs_per_step": support,
        "candidate_pairs_2d_per_step": statistics.mean(k2_pairs),
        "pair_kernel_ms": {"d1": statistics.mean(k1_ms), "d2": statistics.mean(k2_ms)},
        "wall_s_timed": wall,
        "clocks": clk.summary(),
        "e2e": {"value": units_e2e / (e2e / 1e3), "unit": UNIT,
                "h2d_bytes_per_step": int(x.nbytes) * ws,
                "d2h_bytes_per_step": int(mi.nbytes + hx.nbytes) * ws, "ms_per_step": e2e},
        "gpu_launches": launches,
        "autotuned": tuned,
        "roofline": roofline,
    }
    if not args.no_compare and ws == 1:
        pctx = Context(local)  # library defaults for the single-instance calls
        try:
            line["batched_learned_vs_plain"] = compare_plain(ctx, pctx, x, ptr)
        except Exception as exc:
            line["batched_learned_vs_plain"] = {"error": str(exc)[:300]}
        try:
            line["te_batched_learned_vs_plain"] = compare_plain_te(ctx, pctx)
        except Exception as exc:
            line["te_batched_learned_vs_plain"] = {"error": str(exc)[:300]}
        pctx.close()
    if not args.no_compare and ws == 1:
        try:
            line["learned_heldout_c5"] = learned_heldout(ctx)
        except Exception as exc:
            line["learned_heldout_c5"] = {"error": str(exc)[:300]}
    if not args.no_extra and ws == 1:
        try:
            line["other_configs"] = other_configs(ctx)
        except Exception as exc:
            line["other_configs"] = {"error": str(exc)[:300]}
    if not args.no_cpu_baseline and ws == 1:
        try:
            from oracle import oracle as O
            O.build_oracle() if not O.ORACLE_SO.exists() else None
            cores = os.cpu_count() or 1
            # a seeded sample of the job's densities: 6 marginals and 6 joints
            rng_s = np.random.default_rng(5)
            cols = sorted(rng_s.choice(M, 6, replace=False).tolist())
            joints = set()
            while len(joints) < 6:
                i, j = sorted(rng_s.choice(M, 2, replace=False).tolist())
                joints.add((i, j))
            sample = [(c,) for c in cols] + sorted(joints)
            sup = float(sum(c1[c] for c in cols) + sum(cnt[i, j] for i, j in joints))
            rate, dt = cpu_port_sample(x, h, sample, sup)
            line["cpu_baseline"] = {
                "value": rate, "unit": UNIT, "cores": cores, "kind": "port", "seconds": dt,
                "cpu_model": cpu_model(),
                "sample": f"6 1-D marginals (columns {cols}) + 6 2-D joints "
                          f"{sorted(joints)} of the job, N=100k; reference OpenMP algorithm "
                          "restated in C, its linear window scans kept",
                "extrapolated_job_s": support / rate}
        except Exception as exc:  # the baseline is reported, never required
            line["cpu_baseline"] = {"value": None, "error": str(exc)[:200]}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
