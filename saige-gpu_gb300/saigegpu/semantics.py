"""Masked approximation against subset-exact fits on one cohort.

The reference builds every phenotype's GRM from that phenotype's own samples (setgeno over
subSampleInGeno, src/SAIGE/src/SAIGE_fitGLMM_fast.cpp:376-385, 436-495): allele frequencies, the
integer fill, QC and 1/sd are the subset's.  The cohort-GRM engines instead restrict the cohort's
GRM to the subset.  This tool fits the same phenotypes both ways on a synthetic cohort and reports
how far the masked variance components land from the exact ones.

    python -m saigegpu.semantics --n 100000 --m 150000 --phenos 8
"""
import argparse
import json
import time

import numpy as np

from . import native, prep, serve, synth
from .context import GRM_BF16X3_TC, MV_BF16X3_TC, MV_SUBSET_EXACT, Context


def make_specs(ctx, n_pheno, seed, drops=None):
    """Phenotypes of the batching workload: alternating binary / quantitative, masks dropping
    U(5%, 40%) of the cohort (or the given fractions)."""
    n = ctx.n
    rng = np.random.default_rng(seed)
    gvs = [ctx.synth_genetic_value(seed * 7 + k) for k in range(2)]
    specs, info = [], []
    for k in range(n_pheno):
        trait = "binary" if k % 2 == 0 else "quantitative"
        gv = gvs[k % 2] * rng.choice([-1, 1]) + 0.3 * gvs[(k + 1) % 2]
        gv = gv / gv.std()
        drop = rng.uniform(0.05, 0.40) if drops is None else drops[k % len(drops)]
        mask = rng.uniform(size=n) > drop
        S = np.nonzero(mask)[0]
        y, C = synth.simulate_pheno(gv, seed * 100 + k, trait, tau=0.3, prevalence=rng.uniform(0.05, 0.3),
                                    h2=rng.uniform(0.1, 0.6))
        f0 = prep.make_fit0(y[S], C[S], trait, True)
        specs.append(serve.FitSpec(f0, trait, mask=mask, name="pheno%d" % k))
        info.append({"trait": trait, "drop": round(float(1.0 - mask.mean()), 4), "n_sub": int(mask.sum())})
    return specs, info


def compare(ctx, specs, max_columns=1024):
    """Fits specs with the subset-exact engine and with the masked split-BF16 engine (building the
    split-BF16 GRM); returns per-phenotype theta of both and the relative difference."""
    ctx.set_matvec_mode(MV_SUBSET_EXACT)
    t0 = time.perf_counter()
    exact, _ = native.fit_batch(ctx, specs, max_columns=max_columns)
    t_exact = time.perf_counter() - t0
    ctx.set_matvec_mode(MV_BF16X3_TC)
    ctx.grm_build(GRM_BF16X3_TC)
    ctx.set_matvec_mode(MV_BF16X3_TC)
    t0 = time.perf_counter()
    masked, _ = native.fit_batch(ctx, specs, max_columns=max_columns)
    t_masked = time.perf_counter() - t0
    rows = []
    for e, m in zip(exact, masked):
        if isinstance(e, Exception) or isinstance(m, Exception):
            rows.append({"error": str(e if isinstance(e, Exception) else m)})
            continue
        te, tm = np.asarray(e["theta"]), np.asarray(m["theta"])
        rows.append({"tau_exact": [float(x) for x in te], "tau_masked": [float(x) for x in tm],
                     "rel_diff": float(np.max(np.abs(tm - te) / np.abs(te)))})
    return rows, {"exact_s": round(t_exact, 2), "masked_s": round(t_masked, 2)}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=100_000)
    ap.add_argument("--m", type=int, default=150_000)
    ap.add_argument("--miss", type=float, default=0.02)
    ap.add_argument("--seed", type=int, default=1003)
    ap.add_argument("--phenos", type=int, default=8)
    args = ap.parse_args(argv)
    ctx = Context(0)
    ptr, ln = ctx.synth_bed(args.seed, args.n, args.m, args.miss)
    ctx.setgeno_device(ptr, ln, args.n, args.m)
    specs, info = make_specs(ctx, args.phenos, args.seed + 17)
    rows, times = compare(ctx, specs)
    for i, r in zip(info, rows):
        print(json.dumps(dict(i, **r)), flush=True)
    diffs = [r["rel_diff"] for r in rows if "rel_diff" in r]
    print(json.dumps({"n": args.n, "m": args.m, "phenotypes": len(rows), "max_rel_diff": max(diffs),
                      "median_rel_diff": float(np.median(diffs)), "seconds": times}), flush=True)


if __name__ == "__main__":
    main()
