"""tcgen05 paths: BF16 / split-BF16 SYRK and the TF32 GRM.V against the FP64 oracle."""
import numpy as np
import pytest

from oracle import aireml, plink
from saigegpu import GRM_BF16_TC, GRM_BF16X3_TC, GRM_FP32_SIMT, MV_FP32_SIMT, MV_TF32_TC, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cohort(gpu_ctx):
    n, m = 700, 1900  # n % 256 != 0: the last 256-wide column block is partly past n
    bed, _ = synth.synth_bed(31, n, m, 0.01)
    gpu_ctx.setgeno(bed, n, m)
    g = plink.setgeno(bed, n, m, np.arange(1, n + 1), np.ones(n, bool), 0.01, 0.15)
    return gpu_ctx, aireml.DenseGRM(g)


def test_syrk_bf16_tc(cohort):
    ctx, grm = cohort
    ctx.grm_build(GRM_BF16_TC)
    K = ctx.grm_get().astype(np.float64)
    assert np.array_equal(K, K.T)
    err = np.abs(K - grm.K).max()
    assert err < 2e-3, err
    assert np.abs(np.diag(K) - np.diag(grm.K)).max() < 2e-3


def test_syrk_split_bf16_tc(cohort):
    ctx, grm = cohort
    ctx.grm_build(GRM_BF16X3_TC)
    K = ctx.grm_get().astype(np.float64)
    assert np.array_equal(K, K.T)
    err = np.abs(K - grm.K).max() / np.abs(grm.K).max()
    assert err < 2e-5, err


def test_grm_matvec_tf32_tc(cohort):
    ctx, grm = cohort
    ctx.grm_build(GRM_FP32_SIMT)
    rng = np.random.default_rng(0)
    try:
        for k in (1, 31, 64, 130):
            V = rng.standard_normal((grm.n, k))
            ref = grm.K @ V
            ctx.set_matvec_mode(MV_TF32_TC)
            Y = ctx.grm_matmul(V)
            assert np.abs(Y - ref).max() / np.abs(ref).max() < 5e-3, k
    finally:
        ctx.set_matvec_mode(MV_FP32_SIMT)
