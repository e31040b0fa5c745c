"""Variance ratio on the resident GRM (``extractVarianceRatio``, FIT.R:2152-2423).

The reference solves one PCG per marker (``getSigma_G``, FIT.cpp:3394-3398),
marker after marker, adding 10 markers while the CV of the ratios exceeds
``ratioCVcutoff``.  Here each block of markers (30, then 10 at a time) is one
multi-RHS solve on the GPU engine; the per-marker algebra is the reference's:

    G0 flipped to the minor allele, AC = sum(G0)
    G  = G0 - X (X'VX)^-1 X'V G0            (ScoreTest_NULL_Model, FIT.R:579-591)
    var1 = (G'S^-1G - G'S^-1X (X'S^-1X)^-1 X'S^-1G) / AC
    var2 = sum mu(1-mu) g^2 (binary) or sum g^2 (quantitative), g = G / sqrt(AC)
    ratio = var1 / var2;  VR = mean(ratios)

Single-ratio (non-categorical) estimate over the cohort's full sample set.
"""
import numpy as np

from .family import family_of


def _cal_cv(x):
    x = np.asarray(x, np.float64)
    return (x.std(ddof=1) / x.mean()) / len(x)


def variance_ratio(ctx, fit, trait, X, order, num_markers=30, ratio_cv_cutoff=0.001, maxiter=500,
                   tol=1e-5, vr_geno=None):
    """Variance ratio for a fitted null model; returns (VR, per-marker ratios).

    ``fit``: result dict of a null fit (theta, linear_predictors, fitted_values) over all samples;
    ``X``: the design the reference uses (``Xorig`` when covariates are offsets);
    ``order``: indices into the variance-ratio markers (``sg_get_vr_markers``) in test order.
    """
    fam = family_of("binomial" if trait == "binary" else "gaussian")
    eta = np.asarray(fit["linear_predictors"], np.float64)
    mu = np.asarray(fit["fitted_values"], np.float64)
    tau = np.asarray(fit["theta"], np.float64)
    n = len(mu)
    W = (fam.mu_eta(eta) / np.sqrt(fam.variance(mu))) ** 2
    V = mu * (1 - mu) if trait == "binary" else np.full(n, 1.0 / tau[0])
    X = np.asarray(X, np.float64)
    XV = (X * V[:, None]).T
    XXVX_inv = X @ np.linalg.inv(X.T @ (X * V[:, None]))
    SX, _ = ctx.pcg_solve(W, tau, X, maxiter, tol)
    SX = SX.reshape(n, -1)
    XtSX_inv = np.linalg.inv(X.T @ SX)

    def geno(i):
        return (vr_geno[i] if vr_geno is not None else ctx.onesnp_geno(int(i), vr=True)).astype(np.float64)

    ratios = []
    idx = 0
    target = num_markers
    while True:
        block = []
        while len(ratios) + len(block) < target and idx < len(order):
            G0 = geno(order[idx])
            idx += 1
            if G0.sum() / (2 * n) > 0.5:
                G0 = 2 - G0
            AC = G0.sum()
            block.append((G0 - XXVX_inv @ (XV @ G0), AC))
        if block:
            Gm = np.column_stack([b[0] for b in block])
            SG, _ = ctx.pcg_solve(W, tau, Gm, maxiter, tol)
            SG = SG.reshape(n, -1)
            for j, (G, AC) in enumerate(block):
                sg = SG[:, j]
                var1 = (G @ sg - (G @ SX) @ XtSX_inv @ (X.T @ sg)) / AC
                g = G / np.sqrt(AC)
                var2 = float((mu * (1 - mu)) @ (g * g)) if trait == "binary" else float(g @ g)
                ratios.append(var1 / var2)
        if _cal_cv(ratios) > ratio_cv_cutoff and idx < len(order):
            target += 10
            continue
        break
    return float(np.mean(ratios)), np.array(ratios)
