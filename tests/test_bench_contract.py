"""bench.py's host-side contract, without a GPU: the figures it reads from the
committed ncu summaries exist, its clock sampler classifies throttle reasons,
its command line parses, and the reference arm's single-rank rule holds."""
import subprocess
import sys

import pytest

from conftest import ROOT

sys.path.insert(0, str(ROOT))
import bench  # noqa: E402


@pytest.mark.parametrize("profile,key", [
    ("moments2d_mi64x100k_ncu.md", "issue_frac"),
    ("moments2d_mi64x100k_ncu.md", "target_dram_bytes_per_target"),
    ("moments2d_mi64x100k_ncu.md", "edge_fma_pipe_frac"),
    ("moments2d_mi64x100k_ncu.md", "dram_bytes_per_point"),
    ("density3d_sym_te4_ncu.md", "flops_per_pair"),
    ("density3d_sym_te4_ncu.md", "fma_pipe_frac"),
])
def test_profile_figures_present(profile, key):
    v = bench.profile_figure(profile, key)
    assert v is not None and v > 0
    assert bench.ncu_traffic() is not None


def test_clock_summary_reasons(tmp_path):
    s = bench.ClockSampler(0)
    rows = [
        "0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active",
        "0, 2040, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 1200.0, 0x0, Not Active, Not Active, Not Active, Not Active",
        "garbage line",
    ]
    s.f.write("\n".join(rows) + "\n")
    out = s.summary()
    assert out["sm_mhz"] == 2070 and out["sm_max_mhz"] == 2070 and out["samples"] == 3
    assert out["reasons"] == ["sw_power_cap"]
    empty = bench.ClockSampler(0).summary()
    assert empty["samples"] == 0 and empty["reasons"] == ["unsampled"]


def test_peaks_have_a_source():
    gbs, kind = bench.hbm_peak_gbs()
    assert gbs > 1000 and ("measured" in kind or "fallback" in kind)
    tf, note = bench.fp32_peak_tflops(152)
    assert 60 < tf < 90 and "nominal" in note


def test_command_line_parses():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--help"], capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0
    for flag in ("--gpus", "--steps", "--warmup", "--impl", "--coords-file", "--xtc-frames"):
        assert flag in r.stdout


def test_reference_arm_other_ranks_exit_quietly(monkeypatch, capsys):
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    assert bench.dist_env() == (2, 1, 0)

    class Args:
        steps, warmup, gpus = 1, 0, 2
    bench.reference_arm(Args(), None, None)  # rank 1: no work, no output
    assert capsys.readouterr().out == ""
