"""The subset-exact engine at full size (N = 100,000, M = 150,000, 2% missing) against the reference's
own construction of a phenotype's GRM, on the GPU.

The reference runs setgeno over each phenotype's samples (FIT.cpp:376-385, 436-495) and builds
that subset's GRM from them.  Here one context holds the whole cohort in the subset-exact engine
(the genotype matrix G, every subset's QC, fill and 1/sd computed from G's codes per mask); a second
context runs setgeno over the subset's samples only and builds its GRM with the split-BF16 SYRK
(16 significant bits, all four products; within 3e-5 of FP64 in tau at this size) and the split-BF16
GRM.V; the two share nothing but the .bed bytes.  K_S v is also accumulated in FP64 (torch) from
the subset context's own re-packed genotypes and the reference's FP32 standardised values.  Both
engines' K_S v against that FP64 product, and their Sigma_S^-1 v against each other, check the
exact engine's whole chain (subset QC, fill changes, centring, both genotype GEMMs, the finalize)
at the size the benchmark runs.  About a minute and ~150 GB of HBM.
"""
import numpy as np
import pytest

from oracle import plink
from saigegpu import GRM_BF16X3_TC, MV_BF16X3_TC, MV_SUBSET_EXACT, MV_SUBSET_EXACT_F8, Context

pytestmark = pytest.mark.gpu

N, M, MISS, SEED = 100_000, 150_000, 0.02, 1003
DROP = 0.25
K_COLS = 6


def _k_fp64(ctx, V):
    """K V accumulated in FP64 from a context's re-packed genotypes and the reference's FP32
    standardised values (setStdGenoLookUpArr, FIT.cpp:152-159): (1/M) Z'(Z V), Z chunked over markers,
    through torch on the GPU."""
    import torch
    packed = ctx.packed_geno()
    lut = plink.std_lut(ctx.allele_freq(), ctx.invstd())
    n, mq = ctx.n, packed.shape[0]
    dev = torch.device("cuda")
    Vt = torch.from_numpy(np.ascontiguousarray(V, np.float64)).to(dev)
    acc = torch.zeros_like(Vt)
    to_g = torch.tensor([2, 0, 1, 0], dtype=torch.long, device=dev)  # re-packed field -> genotype
    shifts = torch.tensor([0, 2, 4, 6], dtype=torch.uint8, device=dev)
    for m0 in range(0, mq, 4096):
        pk = torch.from_numpy(packed[m0:m0 + 4096]).to(dev)
        f = ((pk.unsqueeze(-1) >> shifts) & 3).reshape(pk.shape[0], -1)[:, :n].long()
        assert not bool((f == 1).any())  # no missing call survives the fill
        z = torch.gather(torch.from_numpy(lut[m0:m0 + 4096]).to(dev).double(), 1, to_g[f])
        acc += z.t() @ (z @ Vt)
        del pk, f, z
    return (acc / mq).cpu().numpy()


def _errs(Y, R):
    return (np.abs(Y - R).max(axis=0) / np.abs(R).max(axis=0),
            np.sqrt(((Y - R) ** 2).mean(axis=0) / (R ** 2).mean(axis=0)))


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
    # setgeno over S: the subset's samples re-packed, and counted for frequencies and QC (the
    # phenotype indicator over the .fam samples)
    sub.setgeno_device(ptr, ln, N, M, sub_1based=(S + 1).astype(np.int32), pheno_mask=mask.astype(np.uint8))
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
    R64 = _k_fp64(sub, V[S])
    ex_max, ex_rms = _errs(Y, R64)
    sp_max, sp_rms = _errs(R, R64)
    print("K_S v against FP64 over setgeno(S): subset-exact engine max %s rms %s; split-BF16 GRM of "
          "setgeno(S) max %s rms %s" % (ex_max, ex_rms, sp_max, sp_rms))
    # the subset-exact engine centres v on S (K_S 1_S = 0), so V's mean of 0.3 costs it nothing:
    # measured 5e-6 max / 4.5e-6 rms.  The split-BF16 GRM of setgeno(S) applies its FP32 K to the
    # mean as well, and the K build's accumulated row-sum error shows (measured 2.3e-4 max / 7.4e-4
    # rms here; 1.4e-5 rms for zero-mean vectors, and its fits' tau within 3e-5 of FP64 at this size)
    assert ex_max.max() < 2e-5 and ex_rms.max() < 2e-5, (ex_max, ex_rms)
    assert sp_max.max() < 1e-3 and sp_rms.max() < 2e-3, (sp_max, sp_rms)
    # the FP16-high / E4M3-low form (15 significant bits of each scaled column)
    whole.set_matvec_mode(MV_SUBSET_EXACT_F8)
    try:
        whole.engine_set_pheno(0, np.ones(N), np.array([1.0, 0.5]), mask)
        Y8 = _run(whole, whole.engine_submit(0, 1, V))[S]
    finally:
        whole.set_matvec_mode(MV_SUBSET_EXACT)
    f8_max, f8_rms = _errs(Y8, R64)
    print("K_S v against FP64, FP16 / E4M3 form: max %s rms %s" % (f8_max, f8_rms))
    assert f8_max.max() < 5e-5 and f8_rms.max() < 5e-5, (f8_max, f8_rms)


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
    err_max, err_rms = _errs(X, Xs)
    print("Sigma_S^-1 b, subset-exact engine against the split-BF16 GRM of setgeno(S): max %s rms %s"
          % (err_max, err_rms))
    assert err_max.max() < 1e-3 and err_rms.max() < 1e-4, (err_max, err_rms)
