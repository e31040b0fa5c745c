"""Variance ratio on the GPU (marker blocks as multi-RHS solves) against the FP64 oracle."""
import numpy as np
import pytest

from oracle import aireml, plink
from saigegpu import GRM_FP32_SIMT, MV_FP32_SIMT, prep, serve, vr

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("trait", ["binary", "quantitative"])
def test_variance_ratio_matches_oracle(gpu_ctx, golden_plink, trait):
    bed, n, m, ph = golden_plink
    rng = np.random.default_rng(5)
    vr_rand = np.unique(rng.integers(0, m, 1000))
    ctx = gpu_ctx
    ctx.set_matvec_mode(MV_FP32_SIMT)
    ctx.setgeno(bed, n, m, vr_random=vr_rand, min_mac_vr=20.0, is_var_ratio=True)
    ctx.grm_build(GRM_FP32_SIMT)
    g = plink.setgeno(bed, n, m, np.arange(1, n + 1), np.ones(n, bool), 0.01, 0.15, vr_rand, 20, True)
    grm = aireml.DenseGRM(g)
    _, _, idx = ctx.vr_markers()
    np.testing.assert_array_equal(idx, g.vr_index)
    for j in (0, len(idx) // 2, len(idx) - 1):
        np.testing.assert_array_equal(ctx.onesnp_geno(j, vr=True), g.vr_codes[j])
    key = "y_binary" if trait == "binary" else "y_quantitative"
    f0 = prep.make_fit0(ph[key], np.column_stack([ph["x1"], ph["x2"]]), trait, True)
    fit = (aireml.glmmkin_binary if trait == "binary" else aireml.glmmkin_quantitative)(grm, f0)
    order = np.random.default_rng(9).permutation(len(idx))
    ref, rref = aireml.variance_ratio(grm, fit, trait, f0["Xorig"], g.vr_codes, order)
    got, rgot = vr.variance_ratio(ctx, fit, trait, f0["Xorig"], order)
    assert len(rgot) == len(rref)
    assert abs(got - ref) / ref < 1e-4, (got, ref)


def test_categorical_variance_ratio_matches_oracle(gpu_ctx, golden_plink):
    """Two MAC categories (isCateVarianceRatio with the fitNULLGLMM defaults): the GPU's marker
    selection equals the oracle's and each category's ratio is within 1e-4 of it."""
    bed, n, m, ph = golden_plink
    rng = np.random.default_rng(5)
    vr_rand = np.unique(rng.integers(0, m, 1000))
    ctx = gpu_ctx
    ctx.set_matvec_mode(MV_FP32_SIMT)
    ctx.set_vr_max_mac(max(vr.CATE_MAX_INCL))
    try:
        ctx.setgeno(bed, n, m, vr_random=vr_rand, min_mac_vr=min(vr.CATE_MIN_EXCL), is_var_ratio=True)
    finally:
        ctx.set_vr_max_mac(-1.0)
    ctx.grm_build(GRM_FP32_SIMT)
    g = plink.setgeno(bed, n, m, np.arange(1, n + 1), np.ones(n, bool), 0.01, 0.15, vr_rand,
                      min(vr.CATE_MIN_EXCL), True, max_mac_vr=max(vr.CATE_MAX_INCL))
    _, mac, idx = ctx.vr_markers()
    np.testing.assert_array_equal(idx, g.vr_index)
    np.testing.assert_array_equal(mac, g.vr_mac)
    grm = aireml.DenseGRM(g)
    f0 = prep.make_fit0(ph["y_binary"], np.column_stack([ph["x1"], ph["x2"]]), "binary", True)
    fit = aireml.glmmkin_binary(grm, f0)
    cats = vr.category_markers(mac)
    orders = [c[np.random.default_rng(9 + k).permutation(len(c))] for k, c in enumerate(cats)]
    ref = aireml.categorical_variance_ratio(grm, fit, "binary", f0["Xorig"], g.vr_codes, orders)
    got = vr.categorical_variance_ratio(ctx, fit, "binary", f0["Xorig"], orders)
    assert len(got) == 2
    for a, b in zip(got, ref):
        assert abs(a - b) / b < 1e-4, (got, ref)
