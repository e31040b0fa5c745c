"""GPU GRM, GRM.V and multi-RHS PCG against the FP64 oracle."""
import numpy as np
import pytest

from oracle import aireml, plink
from saigegpu import MV_FP32_SIMT, MV_FP64_PLAIN, GRM_FP32_SIMT, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cohort(gpu_ctx):
    n, m = 517, 1300
    bed, _ = synth.synth_bed(21, n, m, 0.01)
    gpu_ctx.setgeno(bed, n, m)
    gpu_ctx.grm_build(GRM_FP32_SIMT)
    g = plink.setgeno(bed, n, m, np.arange(1, n + 1), np.ones(n, bool), 0.01, 0.15)
    return gpu_ctx, aireml.DenseGRM(g)


def test_grm_fp32_matches_oracle(cohort):
    ctx, grm = cohort
    K = ctx.grm_get().astype(np.float64)
    assert np.abs(K - K.T).max() == 0.0
    err = np.abs(K - grm.K).max() / np.abs(grm.K).max()
    assert err < 2e-6, err


def test_grm_matmul_more_columns_than_the_engine_holds(cohort):
    ctx, grm = cohort
    V = np.random.default_rng(1).standard_normal((grm.n, 300))
    Y = ctx.grm_matmul(V)
    ref = grm.K @ V
    assert np.abs(Y - ref).max() / np.abs(ref).max() < 5e-6


def test_full_engine_fails_loudly():
    """Held results that nobody consumes make the engine report SG_ERR_STATE instead of waiting."""
    from saigegpu import Context, SaigeGpuError
    n, m = 200, 300
    bed, _ = synth.synth_bed(3, n, m, 0.0)
    with Context(0) as ctx:
        ctx.setgeno(bed, n, m)
        ctx.grm_build(GRM_FP32_SIMT)
        ctx.engine_reserve(32, 1)
        ctx.engine_set_pheno(0, np.full(n, 0.2), np.array([1.0, 0.3]))
        ctx.engine_hold_results(True)
        ids = ctx.engine_submit(0, 1, np.ones((n, 40)), 1, 0.0)
        with pytest.raises(SaigeGpuError):
            for _ in range(10):
                ctx.engine_run(1)
        for i in ids[:5]:
            ctx.engine_cancel(int(i))


def test_grm_matmul(cohort):
    ctx, grm = cohort
    rng = np.random.default_rng(0)
    V = rng.standard_normal((grm.n, 37))
    Y = ctx.grm_matmul(V)
    ref = grm.K @ V
    assert np.abs(Y - ref).max() / np.abs(ref).max() < 5e-6
    y1 = ctx.getCrossprodMatAndKin(V[:, 0].astype(np.float32))
    np.testing.assert_allclose(y1, ref[:, 0], rtol=1e-4, atol=1e-4 * np.abs(ref[:, 0]).max())


@pytest.mark.parametrize("mode", [MV_FP32_SIMT, MV_FP64_PLAIN])
def test_pcg_multi_rhs_matches_oracle(cohort, mode):
    ctx, grm = cohort
    ctx.set_matvec_mode(mode)
    try:
        n = grm.n
        rng = np.random.default_rng(5)
        w = rng.uniform(0.05, 0.25, n)
        tau = np.array([1.0, 0.35])
        B = rng.standard_normal((n, 9))
        X, it = ctx.pcg_solve(w, tau, B, 500, 1e-5)
        Xo, ito = aireml.pcg(grm, w, tau, B, 500, 1e-5, return_iters=True)
        S = np.diag(tau[0] / w) + tau[1] * grm.K
        exact = np.linalg.solve(S, B)
        # both stop on sum r^2 <= 1e-5: compare each to the exact solution and to each other
        for j in range(B.shape[1]):
            assert abs(int(it[j]) - int(ito[j])) <= 1
            assert np.linalg.norm(X[:, j] - exact[:, j]) / np.linalg.norm(exact[:, j]) < 1e-4
            assert np.linalg.norm(X[:, j] - Xo[:, j]) / np.linalg.norm(Xo[:, j]) < 1e-4
    finally:
        ctx.set_matvec_mode(MV_FP32_SIMT)


def test_batched_columns_equal_single_columns(cohort):
    """Continuous batching: a column's result is bit-identical alone or with others."""
    ctx, grm = cohort
    n = grm.n
    rng = np.random.default_rng(6)
    w = rng.uniform(0.05, 0.25, n)
    tau = np.array([1.0, 0.2])
    B = rng.standard_normal((n, 6))
    X, it = ctx.pcg_solve(w, tau, B, 500, 1e-6)
    for j in (0, 3, 5):
        xj, itj = ctx.pcg_solve(w, tau, B[:, j], 500, 1e-6)
        assert itj == it[j]
        assert np.array_equal(xj, X[:, j])


def test_pcg_f32_dropin_and_zero_rhs(cohort):
    ctx, grm = cohort
    n = grm.n
    w = np.full(n, 0.2, np.float32)
    tau = np.array([1.0, 0.3], np.float32)
    b = np.ones(n, np.float32)
    x, it = ctx.getPCG1ofSigmaAndVector(w, tau, b, 500, 1e-5, return_iters=True)
    xo, ito = aireml.pcg(grm, w.astype(np.float64), tau.astype(np.float64), b.astype(np.float64), 500, 1e-5, return_iters=True)
    assert abs(it - ito) <= 1
    np.testing.assert_allclose(x, xo, rtol=1e-4, atol=1e-6)
    x0, it0 = ctx.getPCG1ofSigmaAndVector(w, tau, np.zeros(n, np.float32), 500, 1e-5, return_iters=True)
    assert it0 == 0 and not x0.any()
    x1, it1 = ctx.getPCG1ofSigmaAndVector(w, tau, b, 1, 1e-5, return_iters=True)
    assert it1 == 1


def test_sigma_ops(cohort):
    ctx, grm = cohort
    n = grm.n
    rng = np.random.default_rng(8)
    w = rng.uniform(0.1, 0.3, n).astype(np.float32)
    tau = np.array([1.0, 0.4], np.float32)
    d = ctx.getDiagOfSigma(w, tau)
    np.testing.assert_allclose(d, aireml.get_diag_of_sigma(grm, w.astype(np.float64), tau.astype(np.float64)), rtol=1e-6)
    b = rng.standard_normal(n).astype(np.float32)
    s = ctx.getCrossprod(b, w, tau)
    ref = aireml.get_crossprod(grm, b.astype(np.float64), w.astype(np.float64), tau.astype(np.float64))
    np.testing.assert_allclose(s, ref, rtol=1e-4, atol=1e-4 * np.abs(ref).max())


def test_masked_phenotype_equals_subset_system(cohort):
    """A phenotype slot with a sample mask solves Sigma[S,S] x_S = b_S with the cohort K."""
    ctx, grm = cohort
    n = grm.n
    rng = np.random.default_rng(9)
    mask = (rng.uniform(size=n) > 0.3).astype(np.uint8)
    w = rng.uniform(0.1, 0.3, n)
    tau = np.array([1.0, 0.3])
    b = rng.standard_normal(n)
    ctx.engine_reserve(64, 2)
    ctx.engine_set_pheno(1, w, tau, mask)
    rid = ctx.engine_submit(1, 0, b[:, None], 500, 1e-10)
    res = None
    for _ in range(1000):
        res = ctx.engine_try_fetch(rid[0])
        if res is not None:
            break
        ctx.engine_run()
    x, it = res
    S = np.nonzero(mask)[0]
    Ss = np.diag(tau[0] / w[S]) + tau[1] * grm.K[np.ix_(S, S)]
    exact = np.linalg.solve(Ss, b[S])
    assert np.linalg.norm(x[S] - exact) / np.linalg.norm(exact) < 1e-5
    assert not x[mask == 0].any()
