"""bench.py's measurement arithmetic on the CPU: the GRM.V roofline and the step-width summary."""
import sys

import numpy as np
import pytest

import bench

PEAKS = {"hbm_gbs": 6683.5, "bf16_tflops": 1913.8}
NP = 100096  # N = 100,000 padded to the 128-row tile


def _t(ms_per_launch, cols, launches=10):
    return {"gemm_launches": launches, "gemm_ms": ms_per_launch * launches, "gemm_cols": cols * launches}


def test_wide_split_bf16_launch_is_tensor_bound():
    r = bench.grm_roofline(None, PEAKS, _t(16.5, 448), 100000, NP, "bf16x3", traffic=1.023)
    flops = 3 * 2.0 * NP * NP * 448  # three BF16 products of 2 N^2 per column
    assert r["bound"] == "tensor" and r["unit"] == "TFLOP/s"
    assert r["achieved"] == pytest.approx(flops / 16.5e-3 / 1e12, rel=1e-4)
    assert r["frac"] == pytest.approx(r["achieved"] / 1913.8, rel=1e-3)
    # algorithmic bytes: both BF16 halves of K (4 B per entry) + P halves read and Y written (8 B)
    alg = 4.0 * NP * NP + 8.0 * NP * 448
    assert r["algorithmic_bytes_per_launch"] == pytest.approx(alg)
    assert r["traffic"] == round(1.023 * alg)


def test_narrow_split_bf16_launch_is_hbm_bound():
    r = bench.grm_roofline(None, PEAKS, _t(6.3, 32), 100000, NP, "bf16x3")
    alg = 4.0 * NP * NP + 8.0 * NP * 32
    assert r["bound"] == "hbm" and r["unit"] == "GB/s"
    assert r["achieved"] == pytest.approx(alg / 6.3e-3 / 1e9, rel=1e-4)
    assert r["traffic"] is None


def test_split_tf32_peak_is_half_the_bf16_rate():
    r = bench.grm_roofline(None, PEAKS, _t(60.0, 1024), 100000, NP, "tf32x3")
    assert r["bound"] == "tensor" and r["peak"] == pytest.approx(1913.8 / 2)


def test_step_width_summary():
    # (GRM.V columns, occupied columns, GRM.V ms, step ms, idle ms)
    trace = np.array([[32, 20, 6.0, 6.5, -1], [448, 430, 16.0, 17.0, 0.2], [1024, 1000, 32.0, 33.0, 0.3],
                      [64, 50, 6.2, 6.6, 0.1]], dtype=float)
    s = bench.step_width_summary(trace)
    assert s["steps"] == 4
    assert s["steps_le_128_columns"] == 2
    assert s["grmv_ms_share_steps_le_128_columns"] == pytest.approx((6.0 + 6.2) / (6.0 + 16.0 + 32.0 + 6.2), abs=1e-3)
    assert bench.step_width_summary(np.zeros((0, 5))) is None


def test_defaults_keep_the_timing_rules(monkeypatch):
    monkeypatch.setattr(sys, "argv", ["bench.py"])
    a = bench.parse()
    assert a.gpus == 1 and a.warmup >= 3 and a.steps >= 1
    assert a.mode == "bf16x3" and a.grm == "bf16x3" and a.impl == "ours"
