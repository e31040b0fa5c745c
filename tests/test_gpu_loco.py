"""Leave-one-chromosome-out: GRM products and Get_Coef_LOCO on the GPU against the FP64 oracle."""
import numpy as np
import pytest

from oracle import aireml, plink
from saigegpu import GRM_FP32_SIMT, MV_FP32_SIMT, MV_TF32X3_TC, prep, serve, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cohort(gpu_ctx):
    n, m = 600, 2200
    bed, _ = synth.synth_bed(71, n, m, 0.01)
    ctx = gpu_ctx
    ctx.set_matvec_mode(MV_FP32_SIMT)
    ctx.setgeno(bed, n, m)
    ctx.grm_build(GRM_FP32_SIMT)
    g = plink.setgeno(bed, n, m, np.arange(1, n + 1), np.ones(n, bool), 0.01, 0.15)
    # 22 chromosomes as contiguous blocks of the GRM markers
    mq = g.codes.shape[0]
    chrom = 1 + (np.arange(mq) * 22) // mq
    return ctx, aireml.DenseGRM(g), g, chrom


@pytest.mark.parametrize("mode", [MV_FP32_SIMT, MV_TF32X3_TC])
def test_loco_product(cohort, mode):
    ctx, grm, g, chrom = cohort
    ranges = serve.loco_ranges(chrom)
    b, e = ranges[7]
    ref_grm = aireml.loco_grm(grm, g, b, e)
    V = np.random.default_rng(0).standard_normal((grm.n, 40))
    ctx.set_matvec_mode(mode)
    try:
        ctx.loco_set(b, e)
        Y = ctx.grm_matmul(V)
        ctx.loco_clear()
        Yfull = ctx.grm_matmul(V)
    finally:
        ctx.set_matvec_mode(MV_FP32_SIMT)
    ref = ref_grm.K @ V
    assert np.abs(Y - ref).max() / np.abs(ref).max() < 2e-5
    assert np.abs(Yfull - grm.K @ V).max() / np.abs(ref).max() < 2e-5


def test_loco_coefficients(cohort):
    ctx, grm, g, chrom = cohort
    gv = synth.genetic_value_from_codes(g.codes, 5)
    y, C = synth.simulate_pheno(gv, 8, "binary", tau=0.6, prevalence=0.3)
    f0 = prep.make_fit0(y, C, "binary", True)
    fit = aireml.glmmkin_binary(grm, f0)
    ranges = serve.loco_ranges(chrom)
    sel = {c: ranges[c] for c in (2, 15)}
    got = serve.fit_loco(ctx, [serve.FitSpec(f0, "binary")], [fit], sel, max_columns=256)
    for c, (b, e) in sel.items():
        ref = aireml.get_coef_loco(aireml.loco_grm(grm, g, b, e), f0, fit, "binary")
        r = got[c][0]
        np.testing.assert_allclose(r["coefficients"], ref["alpha"], rtol=1e-5)
        np.testing.assert_allclose(r["linear_predictors"], ref["eta"], rtol=1e-5, atol=1e-7)


def test_loco_bim_range_selects_the_grm_markers(cohort):
    """A chromosome given as .bim markers leaves out the GRM markers inside it: the same products,
    bit for bit, as the GRM-marker range (the GRM markers are the .bim markers passing QC, in order)."""
    ctx, grm, g, chrom = cohort
    ranges = serve.loco_ranges(chrom)
    b, e = ranges[11]
    bim_of_grm = np.nonzero(g.qc_mask)[0]
    V = np.random.default_rng(2).standard_normal((grm.n, 24))
    try:
        ctx.loco_set(b, e)
        Y = ctx.grm_matmul(V)
        # from the .bim marker after the previous chromosome's last GRM marker to the one before
        # the next chromosome's first: .bim markers failing QC at either end change nothing
        lo = int(bim_of_grm[b - 1]) + 1 if b > 0 else 0
        hi = int(bim_of_grm[e + 1]) - 1 if e + 1 < len(bim_of_grm) else len(g.qc_mask) - 1
        ctx.loco_set_bim(lo, hi)
        Yb = ctx.grm_matmul(V)
    finally:
        ctx.loco_clear()
    np.testing.assert_array_equal(Yb, Y)


def test_loco_bim_range_is_checked(cohort):
    """Ranges outside the .bim markers, or holding no GRM marker, are refused; the context stays usable."""
    ctx, grm, g, chrom = cohort
    m = len(g.qc_mask)
    for b, e in ((-1, 5), (5, m), (9, 3)):
        with pytest.raises(Exception):
            ctx.loco_set_bim(b, e)
    dropped = np.nonzero(~g.qc_mask)[0]
    if len(dropped):  # a .bim marker that failed QC alone holds no GRM marker
        with pytest.raises(Exception):
            ctx.loco_set_bim(int(dropped[0]), int(dropped[0]))
    V = np.random.default_rng(4).standard_normal((grm.n, 3))
    np.testing.assert_allclose(ctx.grm_matmul(V), grm.K @ V, rtol=0, atol=2e-5 * np.abs(grm.K @ V).max())
