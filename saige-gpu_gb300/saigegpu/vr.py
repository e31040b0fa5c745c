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

Single ratio (``variance_ratio``; ``variance_ratio_subset`` for a phenotype on its own sample subset in
a subset-exact engine) or one per MAC category (``categorical_variance_ratio``,
isCateVarianceRatio: FIT.R:2245-2280 builds the categories, the loop at :2290-2410 runs the same
estimate per category).  For categories, setgeno selects the markers with
``Context.set_vr_max_mac(max(max_incl))`` and ``min_mac_vr = min(min_excl)`` (FIT.R:1082-1085).
"""
import numpy as np

from .family import family_of


def _cal_cv(x):
    x = np.asarray(x, np.float64)
    return (x.std(ddof=1) / x.mean()) / len(x)


def _ratio_loop(n, solve, geno, fit, trait, X, order, num_markers, ratio_cv_cutoff):
    """The estimate over n samples: ``solve(B)`` returns Sigma^-1 B (n x k), ``geno(i)`` the
    genotypes of variance-ratio marker i."""
    mu = np.asarray(fit["fitted_values"], np.float64)
    tau = np.asarray(fit["theta"], np.float64)
    V = mu * (1 - mu) if trait == "binary" else np.full(n, 1.0 / tau[0])
    X = np.asarray(X, np.float64)
    XV = (X * V[:, None]).T
    XXVX_inv = X @ np.linalg.inv(X.T @ (X * V[:, None]))
    SX = solve(X)
    XtSX_inv = np.linalg.inv(X.T @ SX)
    ratios = []
    idx = 0
    target = num_markers
    while True:
        block = []
        while len(ratios) + len(block) < target and idx < len(order):
            G0 = np.asarray(geno(order[idx]), np.float64)
            idx += 1
            if G0.sum() / (2 * n) > 0.5:
                G0 = 2 - G0
            AC = G0.sum()
            block.append((G0 - XXVX_inv @ (XV @ G0), AC))
        if block:
            SG = solve(np.column_stack([b[0] for b in block]))
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


def _weights(fit, trait):
    fam = family_of("binomial" if trait == "binary" else "gaussian")
    eta = np.asarray(fit["linear_predictors"], np.float64)
    mu = np.asarray(fit["fitted_values"], np.float64)
    return (fam.mu_eta(eta) / np.sqrt(fam.variance(mu))) ** 2


def variance_ratio(ctx, fit, trait, X, order, num_markers=30, ratio_cv_cutoff=0.001, maxiter=500,
                   tol=1e-5, vr_geno=None):
    """Variance ratio for a fitted null model; returns (VR, per-marker ratios).

    ``fit``: result dict of a null fit (theta, linear_predictors, fitted_values) over all samples;
    ``X``: the design the reference uses (``Xorig`` when covariates are offsets);
    ``order``: indices into the variance-ratio markers (``sg_get_vr_markers``) in test order.
    """
    W = _weights(fit, trait)
    tau = np.asarray(fit["theta"], np.float64)
    n = len(W)

    def solve(B):
        return ctx.pcg_solve(W, tau, B, maxiter, tol)[0].reshape(n, -1)

    def geno(i):
        return vr_geno[i] if vr_geno is not None else ctx.onesnp_geno(int(i), vr=True)

    return _ratio_loop(n, solve, geno, fit, trait, X, order, num_markers, ratio_cv_cutoff)


def variance_ratio_subset(ctx, slot, fit, trait, X, mask, order, num_markers=30, ratio_cv_cutoff=0.001,
                          maxiter=500, tol=1e-5):
    """Variance ratio of a phenotype on its own sample subset in a subset-exact engine: the markers
    and genotypes of setgeno over the subset (``Context.engine_subset_vr_markers`` /
    ``engine_subset_geno``; ``order`` indexes the former) and the solves on the subset's GRM through
    phenotype slot ``slot`` (weights set here; the slot must hold no running columns).  ``fit`` and
    ``X`` are over the subset's samples, in cohort order."""
    mask = np.asarray(mask, bool)
    S = np.nonzero(mask)[0]
    W = _weights(fit, trait)
    tau = np.asarray(fit["theta"], np.float64)
    N = len(mask)
    Wc = np.ones(N)
    Wc[S] = W
    ctx.engine_set_pheno(slot, Wc, tau, mask)
    idx, _ = ctx.engine_subset_vr_markers(slot)

    def solve(B):
        B = np.asarray(B, np.float64).reshape(len(S), -1)
        Bc = np.zeros((N, B.shape[1]))
        Bc[S] = B
        ids = ctx.engine_submit(slot, 0, Bc, maxiter, tol)
        out = {}
        while len(out) < len(ids):
            ctx.engine_run()
            for i in ids:
                if int(i) not in out:
                    r = ctx.engine_try_fetch(int(i))
                    if r is not None:
                        out[int(i)] = r[0]
        return np.column_stack([out[int(i)] for i in ids])[S]

    def geno(i):
        return ctx.engine_subset_geno(slot, int(idx[i]))[S]

    return _ratio_loop(len(S), solve, geno, fit, trait, X, order, num_markers, ratio_cv_cutoff)


# default MAC categories of fitNULLGLMM (FIT.R:683-684): 10 < MAC <= 20.5 and MAC > 20.5
CATE_MIN_EXCL = (10.0, 20.5)
CATE_MAX_INCL = (20.5,)


def category_markers(mac, min_excl=CATE_MIN_EXCL, max_incl=CATE_MAX_INCL):
    """Indices of the variance-ratio markers in each MAC category (FIT.R:2245-2260): category i
    holds min_excl[i] < MAC <= max_incl[i]; the last one MAC > min_excl[-1] (and <= max_incl[-1]
    when max_incl has as many entries as there are categories)."""
    mac = np.asarray(mac, np.float64)
    k = len(min_excl)
    cats = []
    for i in range(k - 1):
        cats.append(np.nonzero((mac > min_excl[i]) & (mac <= max_incl[i]))[0])
    if len(max_incl) == k - 1:
        cats.append(np.nonzero(mac > min_excl[k - 1])[0])
    else:
        cats.append(np.nonzero((mac > min_excl[k - 1]) & (mac <= max_incl[k - 1]))[0])
    return cats


def categorical_variance_ratio(ctx, fit, trait, X, orders, num_markers=30, ratio_cv_cutoff=0.001, maxiter=500,
                               tol=1e-5, vr_geno=None):
    """One variance ratio per MAC category; ``orders[k]``: indices into the variance-ratio markers of
    category k in test order (the reference shuffles each category with R's ``sample``).  A category
    with fewer than num_markers markers is an error, as in the reference (FIT.R:2262-2278)."""
    out = []
    for k, order in enumerate(orders):
        if len(order) < num_markers:
            raise ValueError("MAC category %d has %d variance-ratio markers, fewer than %d" % (k + 1, len(order),
                                                                                            num_markers))
        v, _ = variance_ratio(ctx, fit, trait, X, order, num_markers, ratio_cv_cutoff, maxiter, tol, vr_geno)
        out.append(v)
    return out
