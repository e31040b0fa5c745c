"""The subset-exact engine at full size (N = 100,000, M = 150,000, 2% missing) against the reference's
own construction of a phenotype's GRM, on the GPU.

The reference runs setgeno over each phenotype's samples (FIT.cpp:376-385, 436-495) and builds
that subset's GRM from them.  Here one context holds the whole cohort in the subset-exact engine
(the genotype matrix G, every subset's QC, fill and 1/sd computed from G's codes per mask); a second
context runs setgeno over the subset's samples only and builds its GRM with the split-BF16 SYRK
(16 significant bits, all four products; within 3e-5 of FP64 in tau at this size) and the split-BF16
GRM.V.  The two share nothing but the .bed bytes, so agreement of K_S v and of Sigma_S^-1 v at full
size checks the exact engine's whole chain (subset QC, fill changes, centring, both genotype GEMMs,
the finalize) at the size the benchmark runs.  About a minute and ~150 GB of HBM.
"""
import numpy as np
import pytest

from saigegpu import GRM_BF16X3_TC, MV_BF16X3_TC, MV_SUBSET_EXACT, Context

pytestmark = pytest.mark.gpu

N, M, MISS, SEED = 100_000, 150_000, 0.02, 1003
DROP = 0.25
K_COLS = 6


def _run(ctx, ids):
    pending = [int(i) for i in ids]
    out = {}
    for _ in range(100000):
        if not pending:
            break
        ctx.engine_run()
        for i in list(pending):
            r = ctx.engine_try_fetch(i)
            if r is not None:
                out[i] = r[0]
                pending.remove(i)
    assert not pending
    return np.column_stack([out[int(i)] for i in ids])


@pytest.fixture(scope="module")
def two_paths():
    rng = np.random.default_rng(41)
    mask = rng.uniform(size=N) > DROP
    S = np.nonzero(mask)[0]
    whole = Context(0)
    ptr, ln = whole.synth_bed(SEED, N, M, MISS)
    whole.setgeno_device(ptr, ln, N, M)
    whole.set_matvec_mode(MV_SUBSET_EXACT)
    sub = Context(0)
    sub.setgeno_device(ptr, ln, N, M, sub_1based=(S + 1).astype(np.int32))
    sub.grm_build(GRM_BF16X3_TC)
    sub.set_matvec_mode(MV_BF16X3_TC)
    try:
        yield whole, sub, mask, S
    finally:
        sub.close()
        whole.close()


def test_fullsize_subset_product_matches_setgeno_over_subset(two_paths):
    whole, sub, mask, S = two_paths
    rng = np.random.default_rng(3)
    V = rng.standard_normal((N, K_COLS)) + 0.3
    V[~mask] = 0.0
    whole.engine_reserve(64, 1)
    whole.engine_set_pheno(0, np.ones(N), np.array([1.0, 0.5]), mask)
    Y = _run(whole, whole.engine_submit(0, 1, V))[S]
    sub.engine_reserve(64, 1)
    sub.engine_set_pheno(0, np.ones(len(S)), np.array([1.0, 0.5]))
    R = _run(sub, sub.engine_submit(0, 1, V[S]))
    err = np.abs(Y - R).max(axis=0) / np.abs(R).max(axis=0)
    print("K_S v, max |exact - setgeno(S) split-BF16| / max |.| per column:", err)
    # each path carries its vector operand in 16 significant bits (two BF16 halves): the same bound
    # as the small-N tests against FP64
    assert err.max() < 6e-5, err


def test_fullsize_subset_solve_matches_setgeno_over_subset(two_paths):
    whole, sub, mask, S = two_paths
    rng = np.random.default_rng(4)
    W = rng.uniform(0.1, 0.25, size=N)  # binomial weights mu (1 - mu)
    tau = np.array([1.0, 0.4])
    B = rng.standard_normal((N, 3))
    B[~mask] = 0.0
    whole.engine_set_pheno(0, W, tau, mask)
    X = _run(whole, whole.engine_submit(0, 0, B, maxiter=2000, tol=1e-12))[S]
    sub.engine_set_pheno(0, W[S], tau)
    Xs = _run(sub, sub.engine_submit(0, 0, B[S], maxiter=2000, tol=1e-12))
    err = np.abs(X - Xs).max(axis=0) / np.abs(Xs).max(axis=0)
    print("Sigma_S^-1 b, max |exact - setgeno(S) split-BF16| / max |.| per column:", err)
    assert err.max() < 1e-4, err
