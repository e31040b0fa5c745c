"""bench.py's measurement arithmetic on the CPU: the GRM.V roofline and the step-width summary."""
import sys

import numpy as np
import pytest

import bench

PEAKS = {"hbm_gbs": 6792.7, "bf16_tflops": 1929.7, "bf16_tflops_sustained": 1729.4}
NP = 100096  # N = 100,000 padded to the 128-row tile


def _t(ms_per_launch, cols, launches=10):
    return {"gemm_launches": launches, "gemm_ms": ms_per_launch * launches, "gemm_cols": cols * launches}


def test_split_bf16_launch_roofline_is_algorithmic():
    r = bench.grm_roofline(None, PEAKS, _t(16.5, 448), 100000, NP, "bf16x3", traffic=1.023)
    # algorithmic bytes: both BF16 halves of K (4 B per entry) + P halves read and Y written (8 B);
    # algorithmic FLOPs: one product, 2 N^2 per column
    alg = 4.0 * NP * NP + 8.0 * NP * 448
    flops = 2.0 * NP * NP * 448
    assert r["algorithmic_bytes_per_launch"] == pytest.approx(alg)
    assert r["algorithmic_flops_per_launch"] == pytest.approx(flops)
    # at 448 columns the algorithmic HBM time (5.9 ms) exceeds the algorithmic tensor time (5.2 ms)
    assert r["bound"] == "hbm" and r["unit"] == "GB/s"
    assert r["achieved"] == pytest.approx(alg / 16.5e-3 / 1e9, rel=1e-4)
    assert r["frac"] == pytest.approx(r["achieved"] / 6792.7, rel=1e-3)
    assert r["traffic"] == round(1.023 * alg)
    # executed: three BF16 products against the sustained BF16 rate
    ex = r["executed"]
    assert ex["products"] == 3
    assert ex["frac"] == pytest.approx(3 * flops / 16.5e-3 / 1e12 / 1729.4, rel=1e-3)


def test_subset_engine_roofline_counts_both_genotype_gemms():
    mg = 150016
    r = bench.subset_roofline(PEAKS, _t(30.0, 416), NP, mg)
    alg = 2.0 * 2.0 * NP * mg + 8.0 * (NP + mg) * 416
    flops = 2.0 * 2.0 * NP * mg * 416
    assert r["algorithmic_bytes_per_launch"] == pytest.approx(alg)
    assert r["algorithmic_flops_per_launch"] == pytest.approx(flops)
    assert r["bound"] == "tensor" and r["achieved"] == pytest.approx(flops / 30e-3 / 1e12, rel=1e-4)
    assert r["executed"]["frac"] == pytest.approx(2 * flops / 30e-3 / 1e12 / 1729.4, rel=1e-3)


def test_wide_launch_is_tensor_bound_on_algorithmic_flops():
    r = bench.grm_roofline(None, PEAKS, _t(40.0, 1024), 100000, NP, "bf16x3")
    assert r["bound"] == "tensor" and r["unit"] == "TFLOP/s"
    assert r["achieved"] == pytest.approx(2.0 * NP * NP * 1024 / 40e-3 / 1e12, rel=1e-4)
    assert r["peak"] == 1729.4
    assert r["traffic"] is None


def test_split_tf32_peak_is_half_the_bf16_rate():
    r = bench.grm_roofline(None, PEAKS, _t(60.0, 4096), 100000, NP, "tf32x3")
    assert r["bound"] == "tensor" and r["peak"] == pytest.approx(1729.4 / 2)


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
    assert a.mode == "subset" and a.grm == "bf16x3" and a.impl == "ours"
