"""Batched multi-phenotype fits on the GPU engine: oracle parity and alone-vs-in-the-mix identity."""
import numpy as np
import pytest

from oracle import aireml, plink
from saigegpu import GRM_FP32_SIMT, MV_FP32_SIMT, MV_TF32X3_TC, prep, serve, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cohort(gpu_ctx):
    n, m = 640, 1600
    bed, _ = synth.synth_bed(41, n, m, 0.02)
    gpu_ctx.set_matvec_mode(MV_FP32_SIMT)
    gpu_ctx.setgeno(bed, n, m)
    gpu_ctx.grm_build(GRM_FP32_SIMT)
    g = plink.setgeno(bed, n, m, np.arange(1, n + 1), np.ones(n, bool), 0.01, 0.15)
    grm = aireml.DenseGRM(g)
    gv = synth.genetic_value_from_codes(g.codes, 7)
    rng = np.random.default_rng(3)
    specs, refs = [], []
    for k, trait in enumerate(["binary", "quantitative", "binary", "quantitative"]):
        y, C = synth.simulate_pheno(gv, 50 + k, trait, tau=0.6, prevalence=0.25, h2=0.5)
        mask = None if k < 2 else rng.uniform(size=n) > 0.2
        S = np.arange(n) if mask is None else np.nonzero(mask)[0]
        f0 = prep.make_fit0(y[S], C[S], trait, True)
        specs.append(serve.FitSpec(f0, trait, mask=mask))
        sub = aireml.DenseGRM.from_matrix(grm.K[np.ix_(S, S)], grm.m_qc, grm.diag_sum[S])
        refs.append((aireml.glmmkin_binary if trait == "binary" else aireml.glmmkin_quantitative)(sub, f0)
                    if mask is None else None)
    return gpu_ctx, grm, specs, refs


def test_batched_fits_match_oracle(cohort):
    ctx, grm, specs, refs = cohort
    res, jobs = serve.fit_batch(ctx, specs, max_columns=256)
    for r, ref in zip(res, refs):
        assert not isinstance(r, Exception), r
        if ref is not None:
            # tau within 1e-4 relative of the FP64 oracle with the same probes
            np.testing.assert_allclose(r["theta"], ref["theta"], rtol=1e-4)
            np.testing.assert_allclose(r["coefficients"], ref["coefficients"], rtol=1e-4, atol=1e-8)


def test_alone_equals_in_the_mix(cohort):
    ctx, grm, specs, refs = cohort
    mix, _ = serve.fit_batch(ctx, specs, max_columns=256)
    for k in (1, 2):
        alone, _ = serve.fit_batch(ctx, [specs[k]], max_columns=256)
        np.testing.assert_allclose(alone[0]["theta"], mix[k]["theta"], rtol=1e-12)
        np.testing.assert_allclose(alone[0]["linear_predictors"], mix[k]["linear_predictors"], rtol=1e-12, atol=1e-14)


def test_split_tf32_engine_matches_oracle(cohort):
    ctx, grm, specs, refs = cohort
    ctx.set_matvec_mode(MV_TF32X3_TC)
    try:
        res, _ = serve.fit_batch(ctx, specs[:2], max_columns=256)
        for r, ref in zip(res, refs[:2]):
            np.testing.assert_allclose(r["theta"], ref["theta"], rtol=1e-4)
    finally:
        ctx.set_matvec_mode(MV_FP32_SIMT)


def test_serving_stream(cohort):
    ctx, grm, specs, refs = cohort
    arrivals = [(0.02 * i, specs[i % len(specs)]) for i in range(6)]
    done = serve.serve(ctx, arrivals, max_columns=128, max_phenos=3)
    assert len(done) == 6
    assert all(j.error is None for j in done)
    lat = [j.t_done - j.t_arrive for j in done]
    assert min(lat) > 0
