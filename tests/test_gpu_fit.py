"""Trace, AI score and the full AI-REML fit through the GPU drop-ins vs the FP64 oracle."""
import numpy as np
import pytest

from oracle import aireml, plink
from saigegpu import GRM_FP32_SIMT, glmm, prep

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def golden_cohort(gpu_ctx, golden_plink):
    bed, n, m, ph = golden_plink
    gpu_ctx.setgeno(bed, n, m)
    gpu_ctx.grm_build(GRM_FP32_SIMT)
    g = plink.setgeno(bed, n, m, np.arange(1, n + 1), np.ones(n, bool), 0.01, 0.15)
    return gpu_ctx, aireml.DenseGRM(g), ph


def test_trace_and_ai_score(golden_cohort):
    ctx, grm, ph = golden_cohort
    n = grm.n
    fit0 = prep.make_fit0(ph["y_binary"], np.column_stack([ph["x1"], ph["x2"]]), "binary", True)
    mu = 1 / (1 + np.exp(-fit0["linear_predictors"]))
    w = mu * (1 - mu)
    tau = np.array([1.0, 0.3])
    X = fit0["X"]
    Y = fit0["linear_predictors"] + (fit0["y"] - mu) / w
    rc = aireml.get_coefficients(grm, Y, X, w, tau, 500, 1e-5)
    rg = ctx.getCoefficients(Y, X, w, tau, 500, 1e-5)
    np.testing.assert_allclose(rg["alpha"], rc["alpha"], rtol=1e-4)
    np.testing.assert_allclose(rg["Sigma_iY"], rc["Sigma_iY"], rtol=2e-4, atol=1e-5 * np.abs(rc["Sigma_iY"]).max())
    tr, nr = ctx.GetTrace(rc["Sigma_iX"], X, w, tau, rc["cov"], 30, 500, 1e-5, 0.0025)
    tro, nro = aireml.get_trace(grm, rc["Sigma_iX"], X, w, tau, rc["cov"], 30, 500, 1e-5, 0.0025)
    assert nr == nro
    assert abs(tr - tro) / abs(tro) < 1e-4
    a = ctx.getAIScore(Y, X, w, tau, rc["Sigma_iY"], rc["Sigma_iX"], rc["cov"])
    ao = aireml.get_ai_score(grm, Y, X, w, tau, rc["Sigma_iY"], rc["Sigma_iX"], rc["cov"], 30, 500, 1e-5, 0.0025)
    for k in ("YPAPY", "Trace", "AI"):
        assert abs(a[k] - ao[k]) / abs(ao[k]) < 1e-4, k


@pytest.mark.parametrize("trait", ["binary", "quantitative"])
def test_full_fit_matches_oracle(golden_cohort, trait):
    ctx, grm, ph = golden_cohort
    cov = np.column_stack([ph["x1"], ph["x2"]])
    key = "y_binary" if trait == "binary" else "y_quantitative"
    fit0 = prep.make_fit0(ph[key], cov, trait, True)
    if trait == "binary":
        ro = aireml.glmmkin_binary(grm, fit0)
        rg = glmm.glmmkin_binary(ctx, fit0)
    else:
        ro = aireml.glmmkin_quantitative(grm, fit0)
        rg = glmm.glmmkin_quantitative(ctx, fit0)
    rel = np.abs(rg["theta"] - ro["theta"]) / np.abs(ro["theta"])
    print("%s drop-in fit: tau %s oracle %s rel %s" % (trait, rg["theta"], ro["theta"], rel))
    # the drop-ins carry float32 vectors across the boundary, like Rcpp does
    assert rel.max() < 1e-3, (rg["theta"], ro["theta"])
    assert rg["iterations"] == ro["iterations"]
    np.testing.assert_allclose(rg["coefficients"], ro["coefficients"], rtol=1e-3, atol=1e-6)


def test_config1_cpu_runnable_case(gpu_ctx):
    """The reference's CPU-runnable configuration: N=2,000, M=5,000, binary (prevalence 0.2), tau=0.3."""
    from saigegpu import synth
    n, m = 2000, 5000
    bed, codes = synth.synth_bed(1001, n, m, 0.01)
    gpu_ctx.setgeno(bed, n, m)
    gpu_ctx.grm_build(GRM_FP32_SIMT)
    g = plink.setgeno(bed, n, m, np.arange(1, n + 1), np.ones(n, bool), 0.01, 0.15)
    grm = aireml.DenseGRM(g)
    gv = synth.genetic_value_from_codes(g.codes, 1001)
    y, C = synth.simulate_pheno(gv, 1001, "binary", tau=0.3, prevalence=0.2)
    fit0 = prep.make_fit0(y, C, "binary", True)
    ro = aireml.glmmkin_binary(grm, fit0)
    rg = glmm.glmmkin_binary(gpu_ctx, fit0)
    assert rg["iterations"] == ro["iterations"]
    np.testing.assert_allclose(rg["theta"], ro["theta"], rtol=1e-3)
    from saigegpu import serve
    from test_serve_cpu import FakeEngine
    rb, _ = serve.fit_batch(gpu_ctx, [serve.FitSpec(fit0, "binary")], max_columns=128)
    np.testing.assert_allclose(rb[0]["theta"], ro["theta"], rtol=1e-4)
    # the batched driver run in FP64 on the CPU (the oracle's PCG per column) as a second check
    r64, _ = serve.fit_batch(FakeEngine(grm), [serve.FitSpec(fit0, "binary")])
    np.testing.assert_allclose(rb[0]["theta"], r64[0]["theta"], rtol=1e-5)
