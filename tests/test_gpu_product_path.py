"""The product combination end to end: split-BF16 SYRK -> split-BF16 GRM.V -> native batched driver.

Held to the FP64 oracle on the FP64 GRM of the same standardised genotypes (oracle.plink's FP32
LUT values, multiplied in FP64), binary and quantitative traits, tau within 1e-4 relative.
"""
import numpy as np
import pytest

from oracle import aireml, plink
from saigegpu import GRM_BF16X3_TC, MV_BF16X3_TC, MV_FP32_SIMT, native, prep, serve, synth

pytestmark = pytest.mark.gpu

N, M = 4000, 8000


@pytest.fixture(scope="module")
def product_cohort(gpu_ctx):
    bed, _ = synth.synth_bed(2024, N, M, 0.02)
    gpu_ctx.set_matvec_mode(MV_FP32_SIMT)
    gpu_ctx.setgeno(bed, N, M)
    gpu_ctx.grm_build(GRM_BF16X3_TC)
    g = plink.setgeno(bed, N, M, np.arange(1, N + 1), np.ones(N, bool), 0.01, 0.15)
    return gpu_ctx, aireml.DenseGRM(g), g


@pytest.mark.parametrize("trait", ["binary", "quantitative"])
def test_product_path_matches_fp64_oracle(product_cohort, trait):
    ctx, grm, g = product_cohort
    gv = synth.genetic_value_from_codes(g.codes, 31)
    y, C = synth.simulate_pheno(gv, 77, trait, tau=0.3, prevalence=0.1, h2=0.4)
    f0 = prep.make_fit0(y, C, trait, True)
    ref = (aireml.glmmkin_binary if trait == "binary" else aireml.glmmkin_quantitative)(grm, f0)
    ctx.set_matvec_mode(MV_BF16X3_TC)
    try:
        res, _ = native.fit_batch(ctx, [serve.FitSpec(f0, trait)], max_columns=128)
    finally:
        ctx.set_matvec_mode(MV_FP32_SIMT)
    assert not isinstance(res[0], Exception), res[0]
    rel = np.abs(res[0]["theta"] - ref["theta"]) / np.abs(ref["theta"])
    print("%s: tau %s oracle %s rel %s" % (trait, res[0]["theta"], ref["theta"], rel))
    assert rel.max() < 1e-4, (res[0]["theta"], ref["theta"])
    np.testing.assert_allclose(res[0]["coefficients"], ref["coefficients"], rtol=1e-4, atol=1e-7)
