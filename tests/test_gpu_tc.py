"""tcgen05 paths: BF16 / split-BF16 SYRK and the TF32 / split GRM.V against the FP64 oracle."""
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


def _bf16(x):
    """float32 -> bfloat16 (round to nearest, ties to even), returned as float32."""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def test_syrk_split_bf16_tc(cohort):
    ctx, grm = cohort
    ctx.grm_build(GRM_BF16X3_TC)
    K = ctx.grm_get().astype(np.float64)
    assert np.array_equal(K, K.T)
    err = np.abs(K - grm.K).max() / np.abs(grm.K).max()
    assert err < 2e-5, err
    # all four products of Z = Zh + Zl: a marker's Zl takes one value per genotype, so dropping
    # Zl Zl' would shift every off-diagonal entry the same way (~8e-7 RMS here); the kernel's sum
    # must sit on the four-product one, up to its FP32 accumulation (~2e-9)
    bed, _ = synth.synth_bed(31, grm.n, 1900, 0.01)
    g = plink.setgeno(bed, grm.n, 1900, np.arange(1, grm.n + 1), np.ones(grm.n, bool), 0.01, 0.15)
    Z = plink.std_geno(g)
    Zh = _bf16(Z)
    Zl = _bf16(Z - Zh).astype(np.float64)
    Zh = Zh.astype(np.float64)
    K4 = (Zh + Zl).T @ (Zh + Zl) / Z.shape[0]
    lolo = Zl.T @ Zl / Z.shape[0]
    off = ~np.eye(grm.n, dtype=bool)
    rms = lambda a: float(np.sqrt(np.mean(a[off] ** 2)))  # noqa: E731
    assert rms(K - K4) < 0.1 * rms(lolo), (rms(K - K4), rms(lolo))


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


@pytest.mark.parametrize("split", [False, True])
def test_syrk_shape_variants_bit_identical(cohort, split):
    """Single CTAs and CTA pairs (tcgen05 cta_group::2), any raster group: the same K, bit for bit,
    also when the row blocks are odd in number (a pair's second block past n loads zeros)."""
    from saigegpu import TC_SYRK_GROUP, TC_SYRK_PAIR
    ctx, grm = cohort
    prec = GRM_BF16X3_TC if split else GRM_BF16_TC
    prev = ctx.tc_options()
    try:
        for n, m in ((grm.n, 1900), (600, 1300)):  # 6 and 5 row blocks of 128
            if n != grm.n:
                bed, _ = synth.synth_bed(33, n, m, 0.01)
                ctx.setgeno(bed, n, m)
                g = plink.setgeno(bed, n, m, np.arange(1, n + 1), np.ones(n, bool), 0.01, 0.15)
                Kref = aireml.DenseGRM(g).K
            else:
                Kref = grm.K
            ctx.set_tc_option(TC_SYRK_PAIR, 0)
            ctx.set_tc_option(TC_SYRK_GROUP, 16)
            ctx.grm_build(prec)
            K1 = ctx.grm_get()
            tol = 2e-5 * np.abs(Kref).max() if split else 2e-3
            assert np.abs(K1 - Kref).max() < tol
            for pair, group in ((0, 1), (1, 1), (1, 2), (1, 16)):
                ctx.set_tc_option(TC_SYRK_PAIR, pair)
                ctx.set_tc_option(TC_SYRK_GROUP, group)
                ctx.grm_build(prec)
                assert np.array_equal(ctx.grm_get(), K1), (n, pair, group)
    finally:
        ctx.set_tc_options(prev)
        bed, _ = synth.synth_bed(31, grm.n, 1900, 0.01)
        ctx.setgeno(bed, grm.n, 1900)


@pytest.mark.parametrize("mode", ["tf32x3", "bf16x3"])
def test_grmv_shape_variants_bit_identical(cohort, mode):
    """Every tile width of the split GRM.V against FP64, and for split-BF16 every (CTA pair, K slice)
    variant the tuner chooses from, bit for bit."""
    from saigegpu import MV_BF16X3_TC, MV_TF32X3_TC, tune
    ctx, grm = cohort
    ctx.grm_build(GRM_FP32_SIMT)
    Kg = ctx.grm_get().astype(np.float64)  # the resident FP32 K the split halves come from
    rng = np.random.default_rng(3)
    # split TF32: ~21 significant bits per operand (the MMA reads the low halves at TF32
    # precision); split BF16: 16.  Both accumulate in the tensor cores' FP32 over n terms.
    tol = 2e-5 if mode == "tf32x3" else 6e-5
    prev = ctx.grmv_plan()
    variants = tune.GRMV_VARIANTS if mode == "bf16x3" else ((0, 0),)
    try:
        ctx.set_matvec_mode(MV_TF32X3_TC if mode == "tf32x3" else MV_BF16X3_TC)
        # every tile width: split-TF32 pads to multiples of 32; split-BF16 to multiples of 16 (32, 48,
        # 80, 112, 144, 160, 176, 208, 256, 256 here), where the odd multiples of 16 end on half a
        # 32-column epilogue chunk
        for k in (32, 40, 70, 100, 140, 150, 170, 200, 256, 512):
            V = rng.standard_normal((grm.n, k))
            ctx.set_grmv_plan([(1 << 30,) + variants[0]])
            Y1 = ctx.grm_matmul(V)
            ref = Kg @ V
            assert np.abs(Y1 - ref).max() / np.abs(ref).max() < tol, k
            for v in variants[1:]:
                ctx.set_grmv_plan([(1 << 30,) + v])
                assert np.array_equal(ctx.grm_matmul(V), Y1), (k, v)
    finally:
        ctx.set_grmv_plan(prev)
        ctx.set_matvec_mode(MV_FP32_SIMT)


def test_grmv_bf16x3_every_tile_width_and_variant(cohort):
    """Every split-BF16 tile width (multiples of 16 up to 256) launches with every (CTA pair, K slice)
    variant and gives the same product."""
    from saigegpu import MV_BF16X3_TC, tune
    ctx, grm = cohort
    ctx.grm_build(GRM_FP32_SIMT)
    rng = np.random.default_rng(4)
    prev = ctx.grmv_plan()
    try:
        ctx.set_matvec_mode(MV_BF16X3_TC)
        for k in range(16, 513, 16):
            V = rng.standard_normal((grm.n, k))
            ctx.set_grmv_plan([(1 << 30,) + tune.GRMV_VARIANTS[0]])
            Y1 = ctx.grm_matmul(V)
            for v in tune.GRMV_VARIANTS[1:]:
                ctx.set_grmv_plan([(1 << 30,) + v])
                assert np.array_equal(ctx.grm_matmul(V), Y1), (k, v)
    finally:
        ctx.set_grmv_plan(prev)
        ctx.set_matvec_mode(MV_FP32_SIMT)


def test_grmv_bf16x3_switching_modes_keeps_k_exact(cohort):
    """Split BF16 halves are built from the exact K; leaving the mode frees them and K is intact."""
    from saigegpu import MV_BF16X3_TC, MV_TF32X3_TC
    ctx, grm = cohort
    ctx.grm_build(GRM_FP32_SIMT)
    K0 = ctx.grm_get()
    npad = ctx.grm_padded_n()
    V = np.random.default_rng(5).standard_normal((grm.n, 40))
    try:
        ctx.set_matvec_mode(MV_TF32X3_TC)
        ctx.set_matvec_mode(MV_BF16X3_TC)  # halves taken from K = Khi + Klo
        Y_a = ctx.grm_matmul(V)
        used_bf16 = ctx.bytes_in_use()
        ctx.set_matvec_mode(MV_FP32_SIMT)
        assert used_bf16 - ctx.bytes_in_use() >= 4 * npad * npad  # the BF16 halves are released
        assert np.array_equal(ctx.grm_get(), K0)
        ctx.set_matvec_mode(MV_BF16X3_TC)  # halves taken from the FP32 K directly
        assert np.array_equal(ctx.grm_matmul(V), Y_a)
    finally:
        ctx.set_matvec_mode(MV_FP32_SIMT)


# ---------------------------------------------------------------- accumulation bias
# The tensor core rounds each accumulation into TMEM toward zero.  Summed over a whole reduction
# that shrank every product: at N = 20k, M = 30k the split GRM.V products by 2e-5 to 6e-5 relative
# (split TF32 twice that) and the BF16 SYRK's diagonal by ~2e-4, growing linearly with the reduction.
# The kernels drain their accumulators into FP32 registers every 512 bytes of K, which leaves a
# few 1e-7 here (test_gpu_precision_fullsize.py holds the full-size case to FP64).

@pytest.fixture(scope="module")
def cohort20k(gpu_ctx):
    n, m = 20000, 30000
    ptr, ln = gpu_ctx.synth_bed(1003, n, m, 0.02)
    gpu_ctx.setgeno_device(ptr, ln, n, m)
    return gpu_ctx


@pytest.mark.parametrize("mode", ["bf16x3", "tf32x3"])
def test_grmv_products_carry_no_accumulation_bias(cohort20k, mode):
    from saigegpu import MV_BF16X3_TC, MV_FP64_PLAIN, MV_TF32X3_TC
    ctx = cohort20k
    ctx.grm_build(GRM_BF16_TC)
    n = ctx.n
    rng = np.random.default_rng(3)
    V = np.column_stack([rng.choice([-1.0, 1.0], size=(n, 4)), rng.standard_normal((n, 4)), np.ones(n),
                         rng.uniform(0, 1, n)])
    try:
        ctx.set_matvec_mode(MV_FP64_PLAIN)
        Y64 = ctx.grm_matmul(V)
        ctx.set_matvec_mode(MV_BF16X3_TC if mode == "bf16x3" else MV_TF32X3_TC)
        Y = ctx.grm_matmul(V)
    finally:
        ctx.set_matvec_mode(MV_FP32_SIMT)
    bias = ((Y - Y64) * Y64).sum(axis=0) / (Y64 * Y64).sum(axis=0)  # error along each product
    assert np.abs(bias).max() < 2e-6, bias
    rel = np.linalg.norm(Y - Y64, axis=0) / np.linalg.norm(Y64, axis=0)
    assert rel.max() < 5e-5, rel


@pytest.mark.parametrize("split", [False, True])
def test_syrk_diagonal_carries_no_accumulation_bias(cohort20k, split):
    ctx = cohort20k
    ctx.grm_build(GRM_BF16X3_TC if split else GRM_BF16_TC)
    S = np.arange(0, ctx.n, 79)[:256]
    E = np.zeros((ctx.n, len(S)))
    E[S, np.arange(len(S))] = 1.0
    ctx.set_matvec_mode(MV_FP32_SIMT)
    Kss = ctx.grm_matmul(E)[S, np.arange(len(S))]  # K[s, s], read exactly through unit vectors
    ref = ctx.grm_diag()[S] / ctx.dims()["m_qc"]  # exact sum of z^2 over the GRM markers
    rel = Kss / ref - 1.0
    # BF16 operands round to nearest, once per marker and genotype: every sample sees the same
    # roundings, so their mean error does not average out over samples (~1e-5 at M = 30k); without
    # the drains the mean was ~2e-4 low
    assert abs(rel.mean()) < (5e-5 if not split else 5e-6), rel.mean()
    assert np.abs(rel).max() < (4e-4 if not split else 2e-5), np.abs(rel).max()
