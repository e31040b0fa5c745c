"""Autotuner for the tcgen05 kernels' cluster shapes.

The SYRK and the split GRM.V (TF32 or BF16 halves) can run with 1, 2 or 4 CTAs per
thread-block cluster sharing each B tile through TMA multicast (fewer
L2->SM operand bytes per FLOP).  Which size wins depends on N, the number of
right-hand sides and the tile width, so ``tune`` times every variant on the
resident cohort with the library's CUDA-event timers and keeps the fastest.
All variants produce bit-identical results (same accumulation order).
"""
import argparse
import json
import time

import numpy as np

from .context import GRM_BF16_TC, MV_BF16X3_TC, MV_TF32X3_TC


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


# a larger cluster is kept only when it is faster by more than the spread of repeated timings
MARGIN = 0.02


def _pick(times, clusters):
    best = clusters[0]
    for c in clusters[1:]:
        if times[c] < times[best] * (1.0 - MARGIN):
            best = c
    return best


def tune(ctx, ncols=(128, 384, 1024), tune_syrk=True, clusters=(1, 2, 4), mode=MV_TF32X3_TC):
    """Pick the cluster sizes; leaves the GRM built from 8-bit (BF16) genotypes and engine ``mode``
    selected.  For fits, rebuild it with GRM_BF16X3_TC (16-bit genotypes): at N = 100k the 8-bit
    GRM moved binary variance components by up to 1.1e-3 against FP64.

    The SYRK: the smallest cluster within 2% of the fastest.  The GRM.V: each width's times relative
    to the fastest cluster at that width, summed over the widths (each launched as one pass), the
    smallest cluster within 2% of the lowest sum."""
    report = {"syrk": {}, "grmv": {}}
    if tune_syrk:
        for c in clusters:
            report["syrk"][c] = time_syrk(ctx, c)
        best_s = _pick(report["syrk"], clusters)
        ctx.set_tc_clusters(best_s, ctx.get_tc_clusters()[1])
        ctx.grm_build(GRM_BF16_TC)
    ctx.set_matvec_mode(mode)
    ctx.engine_reserve(max(ncols), 1)  # every width in one launch
    totals = {c: 0.0 for c in clusters}
    for k in ncols:
        times = {c: time_grmv(ctx, c, k) for c in clusters}
        for c in clusters:
            report["grmv"][(c, k)] = times[c]
            totals[c] += times[c] / min(times.values())
    best_g = _pick(totals, clusters)
    ctx.set_tc_clusters(ctx.get_tc_clusters()[0], best_g)
    report["chosen"] = ctx.get_tc_clusters()
    return report


def sweep(ctx, ncols=(32, 64, 128, 256, 512, 1024), clusters=(1, 2, 4),
          modes=((MV_BF16X3_TC, "bf16x3"), (MV_TF32X3_TC, "tf32x3"))):
    """Event-timed SYRK and split GRM.V over cluster sizes, tile widths and column counts on the
    resident cohort; yields one dict per measurement (per-launch milliseconds, TFLOP/s, GB/s)."""
    d = ctx.dims()
    n, mq = d["n"], d["m_qc"]
    prev = ctx.get_tc_clusters()
    try:
        for c in clusters:
            ctx.set_tc_clusters(c, prev[1])
            ms = []
            for _ in range(2):
                ctx.grm_build(GRM_BF16_TC)
                ms.append(ctx.build_timing()["syrk_ms"])
            yield {"kernel": "syrk_bf16", "cluster": c, "syrk_ms": [round(x, 2) for x in ms],
                   "tflops": round(n * (n + 1.0) * mq / (min(ms) * 1e-3) / 1e12, 1)}
        ctx.set_tc_clusters(prev[0], prev[1])
        ctx.grm_build(GRM_BF16_TC)
        npad = ctx.grm_padded_n()
        rng = np.random.default_rng(0)
        for mode, name in modes:
            ctx.set_matvec_mode(mode)
            ctx.engine_reserve(max(ncols), 1)
            kbytes = 4.0 if name == "bf16x3" else 8.0
            for k in ncols:
                V = rng.standard_normal((n, k))
                for c in clusters:
                    ctx.set_tc_clusters(prev[0], c)
                    ctx.grm_matmul(V)
                    ctx.engine_reset_timing()
                    ctx.grm_matmul(V)
                    t = ctx.engine_timing()
                    launches = max(1, t["gemm_launches"])
                    ms = t["gemm_ms"] / launches
                    cols = t["gemm_cols"] / launches
                    yield {"kernel": "grmv_" + name, "k": k, "cluster": c, "cols": cols, "ms": round(ms, 3),
                           "GBps": round((kbytes * npad * npad + 12.0 * npad * cols) / (ms * 1e-3) / 1e9, 1),
                           "tflops": round(3 * 2.0 * npad * npad * cols / (ms * 1e-3) / 1e12, 1)}
    finally:
        ctx.set_tc_clusters(*prev)


def main(argv=None):
    """python -m saigegpu.tune [--n N --m M]: the sweep above on a synthetic cohort, JSON lines."""
    from .context import Context
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=100_000)
    ap.add_argument("--m", type=int, default=150_000)
    ap.add_argument("--miss", type=float, default=0.02)
    ap.add_argument("--seed", type=int, default=1003)
    args = ap.parse_args(argv)
    ctx = Context(0)
    ptr, ln = ctx.synth_bed(args.seed, args.n, args.m, args.miss)
    ctx.setgeno_device(ptr, ln, args.n, args.m)
    for row in sweep(ctx):
        print(json.dumps(row), flush=True)


if __name__ == "__main__":
    main()
