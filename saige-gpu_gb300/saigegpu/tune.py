"""Autotuner for the tcgen05 kernels' shapes, from measured times on the resident cohort.

SYRK: single CTAs (128 x 256 tiles) or CTA pairs (tcgen05 cta_group::2, 256 x 256 tiles), and the
raster group (how many row tiles sweep the column blocks together, which sets how many Z panels the
resident tiles share in L2).

Split-BF16 GRM.V: per launch-width bucket, single CTAs or CTA pairs and the K slice per pipeline
stage (64 bytes: twice the stages; 128: half the barrier round trips).  The chosen table goes into
the library (``Context.set_grmv_plan``), which applies it to every later launch.

Subset-exact engine (``MV_SUBSET_EXACT``): per launch-width bucket, single CTAs or CTA pairs and
the K slice of its two genotype GEMMs (``Context.set_subset_plan``).

Every choice gives bit-identical products (same MMA order, same drain length), so tuning never
changes a fit.  The drain length is not tuned: it sets the accumulation bias (the tensor core's
accumulation into TMEM loses magnitude over long chunks), so it stays at the library's 512 bytes.
"""
import argparse
import json
import time

import numpy as np

from .context import GRM_BF16_TC, MV_BF16X3_TC, MV_SUBSET_EXACT, MV_SUBSET_EXACT_F8, TC_SYRK_GROUP, TC_SYRK_PAIR

# launch widths the GRM.V table covers (columns after padding to a tile width)
GRMV_BUCKETS = (32, 64, 96, 128, 160, 224, 320, 448, 640, 1024)
GRMV_VARIANTS = ((0, 128), (0, 64), (1, 128), (1, 64))  # (CTA pair, K slice bytes)
SYRK_VARIANTS = ((1, 8), (0, 16), (1, 16), (1, 32))     # (CTA pair, raster group); the default first
SUBSET_BUCKETS = (32, 64, 128, 192, 256, 384, 512, 768, 1024)
SUBSET_VARIANTS = ((0, 128), (1, 128), (0, 256), (1, 256), (0, 512), (1, 512), (0, 64), (1, 64))  # (CTA pair, K-stage bytes)

# a variant other than the first is kept only when it is faster by more than the spread of
# repeated timings
MARGIN = 0.02


def _pick(times, variants):
    best = variants[0]
    for v in variants[1:]:
        if times[v] < times[best] * (1.0 - MARGIN):
            best = v
    return best


def time_syrk(ctx, pair, group, precision=GRM_BF16_TC, reps=1):
    """Event-timed SYRK of the resident cohort (ms), best of reps."""
    ctx.set_tc_option(TC_SYRK_PAIR, pair)
    ctx.set_tc_option(TC_SYRK_GROUP, group)
    best = float("inf")
    for _ in range(reps):
        ctx.grm_build(precision)
        best = min(best, ctx.build_timing()["syrk_ms"])
    return best


def time_grmv(ctx, ncols, pair, slice_bytes, reps=2, seed=0, V=None):
    """Event-timed split GRM.V launch over ncols columns (ms per launch), best of reps."""
    ctx.set_grmv_plan([(1 << 30, pair, slice_bytes)])  # whatever width the launch pads to
    if V is None:
        V = np.random.default_rng(seed).standard_normal((ctx.n, ncols))
    ctx.grm_matmul(V)
    best = float("inf")
    for _ in range(reps):
        ctx.engine_reset_timing()
        ctx.grm_matmul(V)
        t = ctx.engine_timing()
        best = min(best, t["gemm_ms"] / max(1, t["gemm_launches"]))
    return best


def tune_syrk(ctx, variants=SYRK_VARIANTS):
    """Times the single-product BF16 SYRK per variant and keeps the choice; leaves that GRM built
    (every variant builds the same K)."""
    times = {v: time_syrk(ctx, *v) for v in variants}
    best = _pick(times, variants)
    ctx.set_tc_option(TC_SYRK_PAIR, best[0])
    ctx.set_tc_option(TC_SYRK_GROUP, best[1])
    return {"times_ms": times, "chosen": best}


def tune_grmv(ctx, buckets=GRMV_BUCKETS, variants=GRMV_VARIANTS, mode=MV_BF16X3_TC):
    """Times every variant at every bucket width and installs the per-width plan."""
    ctx.set_matvec_mode(mode)
    ctx.engine_reserve(max(buckets), 1)  # every width in one launch
    table = {}
    plan = []
    rng = np.random.default_rng(0)
    for w in buckets:
        V = rng.standard_normal((ctx.n, w))
        times = {v: time_grmv(ctx, w, *v, V=V) for v in variants}
        best = _pick(times, variants)
        table[w] = {"times_ms": times, "chosen": best}
        plan.append((w, best[0], best[1]))
    ctx.set_grmv_plan(plan)
    return table


def time_subset(ctx, V, pair, slice_bytes, reps=2):
    """Event-timed subset-exact GRM.V launch over V's columns (ms per launch), best of reps."""
    ctx.set_subset_plan([(1 << 30, pair, slice_bytes)])
    ctx.grm_matmul(V)
    best = float("inf")
    for _ in range(reps):
        ctx.engine_reset_timing()
        ctx.grm_matmul(V)
        t = ctx.engine_timing()
        best = min(best, t["gemm_ms"] / max(1, t["gemm_launches"]))
    return best


def tune_subset(ctx, buckets=SUBSET_BUCKETS, variants=SUBSET_VARIANTS, mode=MV_SUBSET_EXACT):
    """Times every (pair, slice) variant of the subset-exact engine ``mode`` at every bucket width on
    the resident cohort and installs the per-width plan; leaves the engine in ``mode``.  The FP16 /
    E4M3 form has 256-byte stages only, so only its CTA-pair choice is timed."""
    ctx.set_matvec_mode(mode)
    if mode == MV_SUBSET_EXACT_F8:
        variants = tuple(v for v in variants if v[1] == 256)
    ctx.engine_reserve(max(buckets), 1)
    table, plan = {}, []
    rng = np.random.default_rng(0)
    for w in buckets:
        V = rng.standard_normal((ctx.n, w))
        times = {v: time_subset(ctx, V, *v) for v in variants}
        best = _pick(times, variants)
        table[w] = {"times_ms": times, "chosen": best}
        plan.append((w, best[0], best[1]))
    ctx.set_subset_plan(plan)
    return table


def tune(ctx, tune_syrk_too=True, mode=MV_BF16X3_TC, grmv=True):
    """SYRK and GRM.V choices from measured times; leaves the single-product BF16 GRM built (rebuild
    it with GRM_BF16X3_TC for fits: at N = 100k the 8-bit GRM moved binary variance components by
    up to 1.1e-3 against FP64) and, when the GRM.V is tuned, the engine in ``mode``."""
    report = {"grmv": {}}
    if tune_syrk_too:
        report["syrk"] = tune_syrk(ctx)
    if grmv:
        report["grmv"] = tune_grmv(ctx, mode=mode)
    report["plan"] = ctx.grmv_plan()
    return report


def report_json(report):
    """The tuner's report with string keys (JSON)."""
    out = {}
    if "syrk" in report:
        out["syrk"] = {"times_ms": {"pair%d_group%d" % k: round(v, 2) for k, v in report["syrk"]["times_ms"].items()},
                       "chosen": {"pair": report["syrk"]["chosen"][0], "group": report["syrk"]["chosen"][1]}}
    out["grmv"] = {str(w): {"times_ms": {"pair%d_slice%d" % k: round(v, 3) for k, v in r["times_ms"].items()},
                            "chosen": {"pair": r["chosen"][0], "slice": r["chosen"][1]}}
                   for w, r in report["grmv"].items()}
    out["plan"] = [list(p) for p in report["plan"]]
    if "subset" in report:
        out["subset"] = {str(w): {"times_ms": {"pair%d_slice%d" % k: round(v, 3) for k, v in r["times_ms"].items()},
                                  "chosen": {"pair": r["chosen"][0], "slice": r["chosen"][1]}}
                         for w, r in report["subset"].items()}
        out["subset_plan"] = [list(p) for p in report["subset_plan"]]
    return out


def main(argv=None):
    """python -m saigegpu.tune [--n N --m M]: the tuner on a synthetic cohort; one JSON report."""
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
    t0 = time.perf_counter()
    rep = tune(ctx)
    rep["subset"] = tune_subset(ctx)
    rep["subset_plan"] = ctx.subset_plan()
    out = report_json(rep)
    out["seconds"] = round(time.perf_counter() - t0, 1)
    out["n"], out["m"] = args.n, args.m
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
