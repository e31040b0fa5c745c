"""Autotuner for the tcgen05 kernels' cluster shapes.

The SYRK and the split GRM.V (TF32 or BF16 halves) can run with 1, 2 or 4 CTAs per
thread-block cluster sharing each B tile through TMA multicast (fewer
L2->SM operand bytes per FLOP).  Which size wins depends on N, the number of
right-hand sides and the tile width, so ``tune`` times every variant on the
resident cohort with the library's CUDA-event timers and keeps the fastest.
All variants produce bit-identical results (same accumulation order).
"""
import time

import numpy as np

from .context import GRM_BF16_TC, MV_TF32X3_TC


def time_syrk(ctx, cluster, precision=GRM_BF16_TC, reps=1):
    _, g = ctx.get_tc_clusters()
    ctx.set_tc_clusters(cluster, g)
    best = float("inf")
    for _ in range(reps):
        t = time.perf_counter()
        ctx.grm_build(precision)  # synchronous: returns when the SYRK has finished
        best = min(best, time.perf_counter() - t)
    return best


def time_grmv(ctx, cluster, ncols, reps=2, seed=0):
    s, _ = ctx.get_tc_clusters()
    ctx.set_tc_clusters(s, cluster)
    V = np.random.default_rng(seed).standard_normal((ctx.n, ncols))
    ctx.grm_matmul(V)
    best = float("inf")
    for _ in range(reps):
        ctx.engine_reset_timing()
        ctx.grm_matmul(V)
        t = ctx.engine_timing()
        best = min(best, t["gemm_ms"] / max(1, t["gemm_launches"]))
    return best / 1e3


def tune(ctx, ncols=(64, 256, 512), tune_syrk=True, clusters=(1, 2, 4), mode=MV_TF32X3_TC):
    """Pick the fastest cluster sizes; leaves the GRM built (BF16) and engine ``mode`` selected."""
    report = {"syrk": {}, "grmv": {}}
    if tune_syrk:
        for c in clusters:
            report["syrk"][c] = time_syrk(ctx, c)
        best_s = min(report["syrk"], key=report["syrk"].get)
        ctx.set_tc_clusters(best_s, ctx.get_tc_clusters()[1])
        ctx.grm_build(GRM_BF16_TC)
    ctx.set_matvec_mode(mode)
    totals = {c: 0.0 for c in clusters}
    for k in ncols:
        for c in clusters:
            t = time_grmv(ctx, c, k)
            report["grmv"][(c, k)] = t
            totals[c] += t
    best_g = min(totals, key=totals.get)
    ctx.set_tc_clusters(ctx.get_tc_clusters()[0], best_g)
    report["chosen"] = ctx.get_tc_clusters()
    return report
