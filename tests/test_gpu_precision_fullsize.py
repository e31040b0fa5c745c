"""Precision of the product path at full size (N = 100,000, M = 150,000, 2% missing) against FP64.

Minutes of GPU time, so it runs only when asked (skipped otherwise):

    SG_FULLSIZE=1 SG_FULLSIZE_OUT=precision.json python -m pytest tests/test_gpu_precision_fullsize.py -m gpu -s

* GRM entries: K[S, S] for 384 seeded samples read from the device -- the split-BF16 tcgen05 SYRK
  (Z = Zh + Zl, all four products; the product path), the single-product BF16 SYRK, the split-BF16
  halves the GRM.V multiplies, and the exact-FP32 CUDA-core SYRK -- against (1/M) sum_m z_im z_jm
  accumulated in FP64, where z are the reference's FP32 standardised genotypes (setStdGenoLookUpArr,
  src/SAIGE/src/SAIGE_fitGLMM_fast.cpp:152-159) of the device's re-packed, imputed genotypes.
  Bounds: a BF16 operand (8 significant bits, round to nearest) is off by at most 2^-8 of itself, so
  each product z_i z_j by at most ~2^-7 of |z_i z_j|; with 16 significant bits (split), ~2^-15.
* tau: null fits (binary, prevalence 0.1, and quantitative) through the batched split-BF16 engine on
  the split-BF16 GRM, against FP64 PCG (FP64 GEMV, one right-hand side per solve) on the exact-FP32
  GRM; the split-BF16 engine on the exact-FP32 GRM separates the GRM.V error from the build error,
  and the single-product BF16 GRM shows what 8-bit genotypes cost.
* variance ratio (extractVarianceRatio, src/SAIGE/R/SAIGE_fitGLMM_fast.R:2152-2423): the same two
  paths for the binary fit.
"""
import json
import os
import time

import numpy as np
import pytest

from oracle import plink

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not os.environ.get("SG_FULLSIZE"), reason="full-size run: set SG_FULLSIZE=1")]

N, M, MISS, SEED = 100_000, 150_000, 0.02, 1003
N_SAMPLED = 384
# 2-bit field of the re-packed GRM genotypes -> genotype (inverse of plink.PACK_CODE; 1 is unused)
FIELD_TO_G = np.array([2, 255, 1, 0], np.uint8)


def _sampled_z(ctx, S):
    """FP32 standardised genotypes (m_qc, |S|) of samples S, from the device's re-packed genotypes."""
    packed = ctx.packed_geno()
    sh = (2 * (S % 4)).astype(np.uint8)
    field = np.right_shift(packed[:, S // 4], sh[None, :]) & 3
    del packed
    g = FIELD_TO_G[field]
    assert (g != 255).all()
    lut = plink.std_lut(ctx.allele_freq(), ctx.invstd())
    return np.take_along_axis(lut, g.astype(np.int64), axis=1)


def _bf16(x):
    """Round float32 to bfloat16 (nearest, ties to even), returned as float32."""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def _entries(ctx, S):
    """K[S, S] as the current GRM.V mode reads it (products with unit vectors are exact)."""
    E = np.zeros((ctx.n, len(S)))
    E[S, np.arange(len(S))] = 1.0
    return ctx.grm_matmul(E)[S, :]


def _err(Kg, Kref, Kabs, rel_bound=2.0 ** -7):
    off = ~np.eye(len(Kref), dtype=bool)
    d = Kg - Kref
    return {"max_abs_offdiag": float(np.abs(d[off]).max()),
            "rms_offdiag": float(np.sqrt(np.mean(d[off] ** 2))),
            "rms_offdiag_of_K": float(np.sqrt(np.mean(Kref[off] ** 2))),
            "max_rel_diag": float(np.max(np.abs(np.diag(d)) / np.abs(np.diag(Kref)))),
            "mean_rel_diag": float(np.mean(np.diag(d) / np.diag(Kref))),
            "max_over_bound": float(np.max(np.abs(d) / (rel_bound * Kabs + 1e-6)))}


def _specs(ctx):
    from saigegpu import prep, serve, synth
    gv = ctx.synth_genetic_value(SEED * 7)
    gv = gv / gv.std()
    specs = []
    for k, (trait, prev) in enumerate([("binary", 0.1), ("binary", 0.1), ("quantitative", None)]):
        y, C = synth.simulate_pheno(gv * (1 if k == 0 else -1), SEED * 100 + k, trait, tau=0.3,
                                    prevalence=prev or 0.2, h2=0.4)
        specs.append(serve.FitSpec(prep.make_fit0(y, C, trait, True), trait, name="pheno%d" % k))
    return specs


def _fits(ctx, specs):
    from saigegpu import native, serve
    t0 = time.perf_counter()
    res, _ = native.fit_batch(ctx, specs, max_columns=serve.columns_for(specs))
    for r in res:
        assert not isinstance(r, Exception), r
    return res, time.perf_counter() - t0


def _vr(ctx, spec, fit):
    from saigegpu import vr
    _, _, idx = ctx.vr_markers()
    order = np.random.default_rng(9).permutation(len(idx))
    v, ratios = vr.variance_ratio(ctx, fit, spec.trait, spec.fit0["Xorig"], order)
    return v, len(ratios)


def test_fullsize_precision_against_fp64():
    from saigegpu import (Context, GRM_BF16_TC, GRM_BF16X3_TC, GRM_FP32_SIMT, MV_BF16X3_TC, MV_FP32_SIMT,
                          MV_FP64_PLAIN)
    rep = {"n": N, "m": M, "missing": MISS, "seed": SEED, "sampled_samples": N_SAMPLED}
    ctx = Context(0)
    try:
        ptr, ln = ctx.synth_bed(SEED, N, M, MISS)
        vr_rand = np.unique(np.random.default_rng(5).integers(0, M, 1000)).astype(np.int32)
        ctx.setgeno_device(ptr, ln, N, M, vr_random=vr_rand, min_mac_vr=20.0, is_var_ratio=True)
        d = ctx.dims()
        rep["m_qc"], rep["m_vr"] = d["m_qc"], d["m_vr"]
        S = np.sort(np.random.default_rng(11).choice(N, N_SAMPLED, replace=False))
        Z32 = _sampled_z(ctx, S)
        Z = Z32.astype(np.float64)
        Kref = Z.T @ Z / d["m_qc"]
        Kabs = np.abs(Z).T @ np.abs(Z) / d["m_qc"]
        # what the tensor-core builds compute with exact arithmetic: Zh Zh' (BF16) and
        # (Zh + Zl)(Zh + Zl)' (split BF16, Zl = bf16(z - Zh)), in FP64
        Zh = _bf16(Z32)
        Zl = _bf16(Z32 - Zh).astype(np.float64)
        Zh = Zh.astype(np.float64)
        K_model_bf16 = Zh.T @ Zh / d["m_qc"]
        K_model_split = (Zh + Zl).T @ (Zh + Zl) / d["m_qc"]
        del Z, Z32, Zh, Zl
        specs = _specs(ctx)

        # single-product BF16 SYRK: 8-bit standardised genotypes
        ctx.grm_build(GRM_BF16_TC)
        ctx.set_matvec_mode(MV_FP32_SIMT)
        Kg = _entries(ctx, S)
        rep["K_bf16_syrk"] = _err(Kg, Kref, Kabs)
        rep["K_bf16_syrk_vs_exact_bf16_products"] = _err(Kg, K_model_bf16, Kabs, 2.0 ** -20)
        ctx.set_matvec_mode(MV_BF16X3_TC)
        bf16_k, _ = _fits(ctx, specs)

        # the product path: split-BF16 SYRK, split-BF16 GRM.V
        ctx.grm_build(GRM_BF16X3_TC)
        ctx.set_matvec_mode(MV_FP32_SIMT)
        Kg = _entries(ctx, S)
        rep["K_split_bf16_syrk"] = _err(Kg, Kref, Kabs, 2.0 ** -15)
        rep["K_split_bf16_syrk_vs_exact_split_products"] = _err(Kg, K_model_split, Kabs, 2.0 ** -20)
        del Kg
        ctx.set_matvec_mode(MV_BF16X3_TC)
        rep["K_split_bf16_syrk_grmv_halves"] = _err(_entries(ctx, S), Kref, Kabs, 2.0 ** -15)
        prod, rep["fits_s_product"] = _fits(ctx, specs)
        vr_prod, rep["vr_markers_product"] = _vr(ctx, specs[0], prod[0])

        # FP64 reference path: exact-FP32 SYRK, FP64 single-RHS PCG
        ctx.grm_build(GRM_FP32_SIMT)
        ctx.set_matvec_mode(MV_FP32_SIMT)
        rep["K_fp32_syrk"] = _err(_entries(ctx, S), Kref, Kabs)
        ctx.set_matvec_mode(MV_BF16X3_TC)
        same_k, _ = _fits(ctx, specs)
        ctx.set_matvec_mode(MV_FP64_PLAIN)
        ref, rep["fits_s_fp64"] = _fits(ctx, specs)
        vr_ref, rep["vr_markers_fp64"] = _vr(ctx, specs[0], ref[0])
    finally:
        ctx.close()

    rep["fits"] = []
    for s, a, b, c, e in zip(specs, prod, same_k, ref, bf16_k):
        rel = lambda x: (np.abs(x["theta"] - c["theta"]) / np.abs(c["theta"])).tolist()  # noqa: E731
        rep["fits"].append({"trait": s.trait, "tau_fp64": c["theta"].tolist(), "tau_product": a["theta"].tolist(),
                            "rel_err_product": rel(a), "rel_err_splitbf16_on_fp32_K": rel(b),
                            "rel_err_on_single_bf16_K": rel(e),
                            "iterations": [int(a["iterations"]), int(c["iterations"])]})
    rep["variance_ratio"] = {"fp64": vr_ref, "product": vr_prod, "rel_err": abs(vr_prod - vr_ref) / abs(vr_ref)}
    print(json.dumps(rep, indent=1))
    out = os.environ.get("SG_FULLSIZE_OUT")
    if out:
        with open(out, "w") as f:
            json.dump(rep, f, indent=1)

    # each product off by at most ~2^-7 (BF16) or ~2^-15 (split BF16) of |z_i z_j|, 1e-6 for the
    # FP32 accumulation; no systematic shrink of the diagonal (the tensor core rounds each TMEM
    # accumulation toward zero; drained accumulation keeps that to a few 1e-7)
    assert rep["K_bf16_syrk"]["max_over_bound"] < 1.0
    assert rep["K_split_bf16_syrk"]["max_over_bound"] < 1.0
    assert rep["K_split_bf16_syrk_grmv_halves"]["max_over_bound"] < 1.0
    assert abs(rep["K_split_bf16_syrk"]["mean_rel_diag"]) < 1e-5
    # the exact-FP32 build, under the reference path, is far closer to FP64 than the BF16 one
    assert rep["K_fp32_syrk"]["max_abs_offdiag"] < 0.01 * rep["K_bf16_syrk"]["max_abs_offdiag"]
    for f in rep["fits"]:
        assert max(f["rel_err_splitbf16_on_fp32_K"]) < 1e-4, f
        assert max(f["rel_err_product"]) < 1e-4, f
    assert rep["variance_ratio"]["rel_err"] < 1e-4
