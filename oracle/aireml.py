"""FP64 oracle of the dense-GRM Sigma^-1 v solves, Hutchinson trace and AI-REML fit.

Every function restates the reference function named in its docstring
(FIT.cpp = src/SAIGE/src/SAIGE_fitGLMM_fast.cpp, FIT.R =
src/SAIGE/R/SAIGE_fitGLMM_fast.R).  Vectors are float64 and the GRM is the
exact dense K = Z'Z / M_qc (the reference applies it implicitly, FIT.cpp:
1669-1708; the product is the same).  Probes come from ``oracle.probes``.
"""
import numpy as np

from . import plink
from .probes import rademacher


class DenseGRM:
    """K = Z'Z / M_qc with its diagonal, from an ``oracle.plink.GenoResult``."""

    def __init__(self, geno, is_diag_one=False, dtype=np.float64):
        z = plink.std_geno(geno).astype(dtype)  # (m_qc, nn)
        self.m_qc = z.shape[0]
        self.n = z.shape[1]
        self.K = (z.T @ z) / self.m_qc
        self.diag_sum = (z * z).sum(axis=0)  # Get_Diagof_StdGeno (FIT.cpp:665-704)
        self.is_diag_one = is_diag_one

    @classmethod
    def from_matrix(cls, K, m_qc, diag_sum=None, is_diag_one=False):
        g = cls.__new__(cls)
        g.K = np.asarray(K, np.float64)
        g.n = g.K.shape[0]
        g.m_qc = m_qc
        g.diag_sum = np.diag(g.K) * m_qc if diag_sum is None else np.asarray(diag_sum, np.float64)
        g.is_diag_one = is_diag_one
        return g

    def matvec(self, b):
        """getCrossprodMatAndKin (FIT.cpp:1953-1981) -> parallelCrossProd / M (FIT.cpp:1669-1708)."""
        return self.K @ b


def get_diag_of_sigma(grm, w, tau):
    """getDiagOfSigma (FIT.cpp:2322-2365): tau1*diagK/M + tau0/W, floored at 1e-4."""
    w = np.asarray(w, np.float64)
    if not grm.is_diag_one:
        d = tau[1] * grm.diag_sum / grm.m_qc + tau[0] / w
    else:
        d = tau[1] + tau[0] / w
    return np.where(d < 1e-4, 1e-4, d)


def get_crossprod(grm, b, w, tau):
    """getCrossprod (FIT.cpp:2397-2425): tau0*b/W + tau1*K b (K skipped when tau1 == 0)."""
    w = np.asarray(w, np.float64)
    wb = b / (w if b.ndim == 1 else w[:, None])
    if tau[1] == 0:
        return tau[0] * wb
    return tau[0] * wb + tau[1] * grm.matvec(b)


def pcg(grm, w, tau, B, maxiter=500, tol=1e-5, return_iters=False):
    """getPCG1ofSigmaAndVector (FIT.cpp:2593-2809), Jacobi preconditioner.

    ``B`` may hold several right-hand sides as columns; each column runs the
    reference's loop on its own (frozen once its sum r^2 <= tol or it reaches
    maxiter), so a column's result is the single-RHS result.
    """
    B = np.asarray(B, np.float64)
    single = B.ndim == 1
    if single:
        B = B[:, None]
    minv = 1.0 / get_diag_of_sigma(grm, w, tau)
    X = np.zeros_like(B)
    R = B.copy()
    Z = minv[:, None] * R
    P = Z.copy()
    sumr2 = (R * R).sum(axis=0)
    iters = np.zeros(B.shape[1], dtype=np.int64)
    active = (sumr2 > tol) & (iters < maxiter)
    while active.any():
        cols = np.nonzero(active)[0]
        p = P[:, cols]
        ap = get_crossprod(grm, p, w, tau)
        rz = (R[:, cols] * Z[:, cols]).sum(axis=0)
        a = rz / (p * ap).sum(axis=0)
        X[:, cols] += a * p
        r1 = R[:, cols] - a * ap
        z1 = minv[:, None] * r1
        bet = (z1 * r1).sum(axis=0) / rz
        P[:, cols] = z1 + bet * p
        Z[:, cols] = z1
        R[:, cols] = r1
        iters[cols] += 1
        sumr2[cols] = (r1 * r1).sum(axis=0)
        active = (sumr2 > tol) & (iters < maxiter)
    out = X[:, 0] if single else X
    return (out, iters) if return_iters else out


def cal_cv(x):
    """calCV (FIT.cpp:3104-3110): (sd/mean)/n with the n-1 standard deviation."""
    x = np.asarray(x, np.float64)
    return (x.std(ddof=1) / x.mean()) / len(x)


def _p_apply(sigma_i_v, Sigma_iX, cov, v):
    # P v = Sigma^-1 v - Sigma^-1 X cov (Sigma^-1 X)' v   (FIT.cpp:3139)
    return sigma_i_v - Sigma_iX @ (cov @ (Sigma_iX.T @ v))


def get_trace(grm, Sigma_iX, X, w, tau, cov, nrun, maxiter, tol, cutoff, seed=200,
              quantitative=False, stats=None):
    """GetTrace (FIT.cpp:3113-3160) / GetTrace_q (FIT.cpp:3409-3472).

    Probes are solved in blocks (30 first, then +10 while the CV exceeds the
    cutoff), each block as one multi-RHS PCG.  Returns the trace (binary) or
    (tr(P), tr(PK)) (quantitative).
    """
    n = grm.n
    t1, t0 = [], []
    start, end = 0, nrun
    while True:
        U = np.stack([rademacher(seed, i, n, getattr(grm, "probe_index", None)) for i in range(start, end)],
                     axis=1)
        Su, it = pcg(grm, w, tau, U, maxiter, tol, return_iters=True)
        if stats is not None:
            stats.append(("trace", U.shape[1], it))
        Pu = _p_apply(Su, Sigma_iX, cov, U)
        Au = grm.matvec(U)
        t1.extend((Au * Pu).sum(axis=0))
        t0.extend((U * Pu).sum(axis=0))
        cv1 = cal_cv(t1)
        cv0 = cal_cv(t0) if quantitative else 0.0
        if cv1 > cutoff or (quantitative and cv0 > cutoff):
            start, end = end, end + 10
            continue
        break
    if quantitative:
        return np.array([np.mean(t0), np.mean(t1)]), len(t1)
    return float(np.mean(t1)), len(t1)


def _inv_sympd(A):
    """inv_sympd(symmatu(A)) with the pinv fallback (FIT.cpp:3183-3190)."""
    A = np.triu(A) + np.triu(A, 1).T
    try:
        L = np.linalg.cholesky(A)
        Li = np.linalg.inv(L)
        return Li.T @ Li
    except np.linalg.LinAlgError:
        return np.linalg.pinv(A)


def get_coefficients(grm, Y, X, w, tau, maxiter, tol, stats=None):
    """getCoefficients (FIT.cpp:3167-3199): Y and the X columns solved together."""
    B = np.column_stack([Y, X])
    S, it = pcg(grm, w, tau, B, maxiter, tol, return_iters=True)
    if stats is not None:
        stats.append(("coef", B.shape[1], it))
    Sigma_iY, Sigma_iX = S[:, 0], S[:, 1:]
    cov = _inv_sympd(X.T @ Sigma_iX)
    alpha = cov @ (Sigma_iX.T @ Y)
    eta = Y - tau[0] * (Sigma_iY - Sigma_iX @ alpha) / w
    return dict(Sigma_iY=Sigma_iY, Sigma_iX=Sigma_iX, cov=cov, alpha=alpha, eta=eta)


def get_ai_score(grm, Y, X, w, tau, Sigma_iY, Sigma_iX, cov, nrun, maxiter, tol, cutoff,
                 seed=200, stats=None):
    """getAIScore (FIT.cpp:3279-3295)."""
    PY = Sigma_iY - Sigma_iX @ (cov @ (Sigma_iX.T @ Y))
    APY = grm.matvec(PY)
    YPAPY = float(PY @ APY)
    trace, nprobe = get_trace(grm, Sigma_iX, X, w, tau, cov, nrun, maxiter, tol, cutoff, seed,
                              stats=stats)
    S, it = pcg(grm, w, tau, APY, maxiter, tol, return_iters=True)
    if stats is not None:
        stats.append(("papy", 1, it))
    # the reference projects the solved vector: PAPY_1 - Sigma_iX cov (Sigma_iX' PAPY_1)
    # (FIT.cpp:3290-3291), not Sigma_iX' APY as P APY would have it
    PAPY = _p_apply(S, Sigma_iX, cov, S)
    AI = float(APY @ PAPY)
    return dict(YPAPY=YPAPY, Trace=trace, PY=PY, AI=AI, nprobe=nprobe)


def get_ai_score_q(grm, Y, X, w, tau, Sigma_iY, Sigma_iX, cov, nrun, maxiter, tol, cutoff,
                   seed=200, stats=None):
    """getAIScore_q (FIT.cpp:3479-3531): cov recomputed, 2x2 AI with A0 = I."""
    cov1 = _inv_sympd(X.T @ Sigma_iX)
    PY = Sigma_iY - Sigma_iX @ (cov1 @ (Sigma_iX.T @ Y))
    APY = grm.matvec(PY)
    YPAPY = float(PY @ APY)
    A0PY = PY
    YPA0PY = float(PY @ A0PY)
    trace, nprobe = get_trace(grm, Sigma_iX, X, w, tau, cov1, nrun, maxiter, tol, cutoff, seed,
                              quantitative=True, stats=stats)
    S, it = pcg(grm, w, tau, np.column_stack([A0PY, APY]), maxiter, tol, return_iters=True)
    if stats is not None:
        stats.append(("papy", 2, it))
    # as in getAIScore, the projection acts on the solved vectors (FIT.cpp:3507-3508, 3513-3514)
    PA0PY = _p_apply(S[:, 0], Sigma_iX, cov1, S[:, 0])
    PAPY = _p_apply(S[:, 1], Sigma_iX, cov1, S[:, 1])
    AI = np.array([[A0PY @ PA0PY, A0PY @ PAPY], [A0PY @ PAPY, APY @ PAPY]])
    return dict(YPAPY=YPAPY, YPA0PY=YPA0PY, Trace=trace, PY=PY, AI=AI, nprobe=nprobe)


def fitglmmai_rpcg(grm, Y, X, w, tau, Sigma_iY, Sigma_iX, cov, nrun, maxiter, tol_pcg, tol,
                   cutoff, seed=200, stats=None):
    """fitglmmaiRPCG (FIT.cpp:3302-3341): binary tau1 Newton step with step-halving."""
    re = get_ai_score(grm, Y, X, w, tau, Sigma_iY, Sigma_iX, cov, nrun, maxiter, tol_pcg, cutoff,
                      seed, stats)
    dtau = (re["YPAPY"] - re["Trace"]) / re["AI"]
    tau0 = np.array(tau, np.float64)
    t = tau0.copy()
    t[1] = tau0[1] + dtau
    t[t < tol] = 0.0
    step = 1.0
    while t[1] < 0.0:
        step *= 0.5
        t[1] = tau0[1] + step * dtau
    t[t < tol] = 0.0
    return t, re


def fitglmmai_rpcg_q(grm, Y, X, w, tau, Sigma_iY, Sigma_iX, cov, nrun, maxiter, tol_pcg, tol,
                     cutoff, seed=200, stats=None):
    """fitglmmaiRPCG_q (FIT.cpp:3610-3662): 2x2 Newton step, GMMAT zeroing, step-halving."""
    tau0 = np.array(tau, np.float64)
    zero = tau0 < tol
    re = get_ai_score_q(grm, Y, X, w, tau0, Sigma_iY, Sigma_iX, cov, nrun, maxiter, tol_pcg,
                        cutoff, seed, stats)
    score = np.array([re["YPA0PY"] - re["Trace"][0], re["YPAPY"] - re["Trace"][1]])
    dtau = np.linalg.solve(re["AI"], score)
    t = tau0 + dtau
    t[zero & (t < tol)] = 0.0
    step = 1.0
    while t[0] < 0.0 or t[1] < 0.0:
        step *= 0.5
        t = tau0 + step * dtau
        t[zero & (t < tol)] = 0.0
    t[t < tol] = 0.0
    return t, re


# ---------------------------------------------------------------- R driver

class Binomial:
    """R binomial(link = "logit") family (C_logit_linkinv / C_logit_mu_eta)."""
    name = "binomial"
    _EPS = np.finfo(np.float64).eps
    _THRESH = 30.0

    def linkinv(self, eta):
        tmp = np.where(eta < -self._THRESH, self._EPS,
                       np.where(eta > self._THRESH, 1.0 / self._EPS, np.exp(np.clip(eta, -700, 700))))
        return tmp / (1.0 + tmp)

    def mu_eta(self, eta):
        opexp = 1.0 + np.exp(np.clip(eta, -700, 700))
        return np.where((eta > self._THRESH) | (eta < -self._THRESH), self._EPS,
                        np.exp(np.clip(eta, -700, 700)) / (opexp * opexp))

    def variance(self, mu):
        return mu * (1.0 - mu)


class Gaussian:
    """R gaussian(link = "identity") family."""
    name = "gaussian"

    def linkinv(self, eta):
        return np.asarray(eta, np.float64).copy()

    def mu_eta(self, eta):
        return np.ones_like(eta, dtype=np.float64)

    def variance(self, mu):
        return np.ones_like(mu, dtype=np.float64)


def get_coef(grm, y, X, tau, family, alpha0, eta0, offset, maxiter_pcg, tol_pcg, maxiter,
             stats=None):
    """Get_Coef (FIT.R:2-35): IRLS working vector and weights around getCoefficients."""
    tol_coef = 0.1
    mu = family.linkinv(eta0)
    mu_eta = family.mu_eta(eta0)
    Y = eta0 - offset + (y - mu) / mu_eta
    sqrtW = mu_eta / np.sqrt(family.variance(mu))
    W = sqrtW ** 2
    for _ in range(maxiter):
        rc = get_coefficients(grm, Y, X, W, tau, maxiter_pcg, tol_pcg, stats)
        alpha = rc["alpha"]
        eta = rc["eta"] + offset
        mu = family.linkinv(eta)
        mu_eta = family.mu_eta(eta)
        Y = eta - offset + (y - mu) / mu_eta
        sqrtW = mu_eta / np.sqrt(family.variance(mu))
        W = sqrtW ** 2
        if np.max(np.abs(alpha - alpha0) / (np.abs(alpha) + np.abs(alpha0) + tol_coef)) < tol_coef:
            break
        alpha0 = alpha
    return dict(Y=Y, alpha=alpha, eta=eta, W=W, cov=rc["cov"], sqrtW=sqrtW,
                Sigma_iY=rc["Sigma_iY"], Sigma_iX=rc["Sigma_iX"], mu=mu)


def glmmkin_binary(grm, fit0, tol=0.02, maxiter=20, nrun=30, tol_pcg=1e-5, maxiter_pcg=500,
                   trace_cv_cutoff=0.0025, tau_init=(0.0, 0.0), seed=200, stats=None):
    """glmmkin.ai_PCG_Rcpp_Binary (FIT.R:79-304), without LOCO.

    ``fit0`` holds the glm fit: y, X, offset, linear_predictors, coefficients.
    """
    fam = Binomial()
    y, X = fit0["y"], fit0["X"]
    n = len(y)
    offset = fit0.get("offset")
    offset = np.zeros(n) if offset is None else np.asarray(offset, np.float64)
    eta = np.asarray(fit0["linear_predictors"], np.float64)
    alpha0 = np.asarray(fit0["coefficients"], np.float64)
    eta0 = eta
    tau = np.array([1.0, 0.0])
    fixtau = np.array([1, 0])
    if tau_init[1] == 0:
        tau[1] = 0.1
    else:
        tau[1] = tau_init[1]
    tau0 = tau.copy()
    rc = get_coef(grm, y, X, tau, fam, alpha0, eta0, offset, maxiter_pcg, tol_pcg, maxiter, stats)
    re = get_ai_score(grm, rc["Y"], X, rc["W"], tau, rc["Sigma_iY"], rc["Sigma_iX"], rc["cov"],
                      nrun, maxiter_pcg, tol_pcg, trace_cv_cutoff, seed, stats)
    tau[1] = max(0.0, tau0[1] + tau0[1] ** 2 * (re["YPAPY"] - re["Trace"]) / n)
    it_used = 0
    for i in range(1, maxiter + 1):
        it_used = i
        alpha0 = rc["alpha"]
        tau0 = tau.copy()
        eta0 = eta
        rc = get_coef(grm, y, X, tau, fam, alpha0, eta0, offset, maxiter_pcg, tol_pcg, maxiter, stats)
        tau, _ = fitglmmai_rpcg(grm, rc["Y"], X, rc["W"], tau, rc["Sigma_iY"], rc["Sigma_iX"],
                                rc["cov"], nrun, maxiter_pcg, tol_pcg, tol, trace_cv_cutoff, seed,
                                stats)
        alpha, eta = rc["alpha"], rc["eta"]
        if tau[1] == 0:
            break
        if np.max(np.abs(tau - tau0) / (np.abs(tau) + np.abs(tau0) + tol)) < tol:
            break
        if np.max(tau) > tol ** (-2):
            it_used = maxiter
            break
    rc = get_coef(grm, y, X, tau, fam, alpha, eta, offset, maxiter_pcg, tol_pcg, maxiter, stats)
    return dict(theta=tau, coefficients=rc["alpha"], linear_predictors=rc["eta"],
                fitted_values=rc["mu"], Y=rc["Y"], residuals=y - rc["mu"], cov=rc["cov"],
                converged=it_used < maxiter, iterations=it_used)


def glmmkin_quantitative(grm, fit0, tol=0.02, maxiter=20, nrun=30, tol_pcg=1e-5, maxiter_pcg=500,
                         trace_cv_cutoff=0.0025, tau_init=(0.0, 0.0), seed=200, stats=None):
    """glmmkin.ai_PCG_Rcpp_Quantitative (FIT.R:309-549), without LOCO."""
    fam = Gaussian()
    y, X = fit0["y"], fit0["X"]
    n = len(y)
    offset = fit0.get("offset")
    offset = np.zeros(n) if offset is None else np.asarray(offset, np.float64)
    eta = np.asarray(fit0["linear_predictors"], np.float64)
    mu = fam.linkinv(eta)
    Y = eta - offset + (y - mu) / fam.mu_eta(eta)
    alpha = np.asarray(fit0["coefficients"], np.float64)
    alpha0 = alpha
    eta0 = eta
    tau = np.zeros(2)
    if sum(tau_init) == 0:
        tau[:] = [1.0, 0.0]
        if abs(np.var(Y, ddof=1)) < 0.1:
            raise ValueError("variance of the phenotype is much smaller than 1")
    else:
        tau[:] = tau_init
    tau0 = tau.copy()
    rc = get_coef(grm, y, X, tau, fam, alpha0, eta0, offset, maxiter_pcg, tol_pcg, maxiter, stats)
    re = get_ai_score_q(grm, rc["Y"], X, rc["W"], tau, rc["Sigma_iY"], rc["Sigma_iX"], rc["cov"],
                        nrun, maxiter_pcg, tol_pcg, trace_cv_cutoff, seed, stats)
    tau[1] = max(0.0, tau0[1] + tau0[1] ** 2 * (re["YPAPY"] - re["Trace"][1]) / n)
    tau[0] = max(0.0, tau0[0] + tau0[0] ** 2 * (re["YPA0PY"] - re["Trace"][0]) / n)
    it_used = 0
    for i in range(1, maxiter + 1):
        it_used = i
        alpha0 = alpha
        tau0 = tau.copy()
        eta0 = eta
        rc = get_coef(grm, y, X, tau, fam, alpha0, eta0, offset, maxiter_pcg, tol_pcg, maxiter, stats)
        tau, _ = fitglmmai_rpcg_q(grm, rc["Y"], X, rc["W"], tau, rc["Sigma_iY"], rc["Sigma_iX"],
                                  rc["cov"], nrun, maxiter_pcg, tol_pcg, tol, trace_cv_cutoff, seed,
                                  stats)
        alpha, eta = rc["alpha"], rc["eta"]
        if tau[0] <= 0:
            raise ValueError("the first variance component parameter estimate is 0")
        if tau[1] <= 0:
            break
        if np.max(np.abs(tau - tau0) / (np.abs(tau) + np.abs(tau0) + tol)) < tol:
            break
        if np.max(tau) > tol ** (-2):
            it_used = maxiter
            break
    rc = get_coef(grm, y, X, tau, fam, alpha, eta, offset, maxiter_pcg, tol_pcg, maxiter, stats)
    return dict(theta=tau, coefficients=rc["alpha"], linear_predictors=rc["eta"],
                fitted_values=rc["mu"], Y=rc["Y"], residuals=y - rc["mu"], cov=rc["cov"],
                converged=it_used < maxiter, iterations=it_used)


def score_null_model(mu, mu2, y, X):
    """ScoreTest_NULL_Model (FIT.R:579-591): XV, XVX, XXVX_inv, ... of the covariate projection."""
    V = np.asarray(mu2, np.float64)
    XV = (X * V[:, None]).T
    XVX = X.T @ (X * V[:, None])
    XVX_inv = np.linalg.inv(XVX)
    XXVX_inv = X @ XVX_inv
    return dict(XV=XV, XVX=XVX, XXVX_inv=XXVX_inv, XVX_inv=XVX_inv, V=V)


def variance_ratio(grm, fit, trait, X, vr_geno, order, num_markers=30, ratio_cv_cutoff=0.001,
                   maxiter=500, tol=1e-5):
    """extractVarianceRatio (FIT.R:2152-2423), single (non-categorical) ratio, dense GRM.

    ``vr_geno``: (m_vr, n) genotypes 0/1/2 of the variance-ratio markers (missing already filled,
    ``Get_OneSNP_Geno_forVarRatio``); ``order``: the marker order (the reference draws it with R's
    ``sample``).  X is the fit's design (``Xorig`` when covariates are offsets).
    """
    fam = Binomial() if trait == "binary" else Gaussian()
    eta = np.asarray(fit["linear_predictors"], np.float64)
    mu = np.asarray(fit["fitted_values"], np.float64)
    tau = np.asarray(fit["theta"], np.float64)
    mu_eta = fam.mu_eta(eta)
    W = (mu_eta / np.sqrt(fam.variance(mu))) ** 2
    mu2 = mu * (1 - mu) if trait == "binary" else np.full(len(mu), 1.0 / tau[0])
    noK = score_null_model(mu, mu2, None, X)
    SX = pcg(grm, W, tau, X, maxiter, tol)
    XtSX_inv = np.linalg.inv(X.T @ SX)
    n = len(mu)
    ratios = []
    idx = 0
    target = num_markers
    while True:
        while len(ratios) < target and idx < len(order):
            G0 = vr_geno[order[idx]].astype(np.float64)
            idx += 1
            if G0.sum() / (2 * n) > 0.5:
                G0 = 2 - G0
            AC = G0.sum()
            G = G0 - noK["XXVX_inv"] @ (noK["XV"] @ G0)
            g = G / np.sqrt(AC)
            SG = pcg(grm, W, tau, G, maxiter, tol)
            var1 = (G @ SG - (G @ SX) @ XtSX_inv @ (X.T @ SG)) / AC
            var2 = float((mu * (1 - mu)) @ (g * g)) if trait == "binary" else float(g @ g)
            ratios.append(var1 / var2)
        cv = cal_cv(ratios)
        if cv > ratio_cv_cutoff and idx < len(order):
            target += 10
            continue
        break
    return float(np.mean(ratios)), np.array(ratios)


def categorical_variance_ratio(grm, fit, trait, X, vr_geno, orders, num_markers=30, ratio_cv_cutoff=0.001,
                               maxiter=500, tol=1e-5):
    """extractVarianceRatio with isCateVarianceRatio (FIT.R:2245-2410): the single-ratio estimate
    run once per MAC category over that category's markers, in ``orders[k]``."""
    out = []
    for order in orders:
        if len(order) < num_markers:
            raise ValueError("a MAC category has fewer than %d variance-ratio markers" % num_markers)
        out.append(variance_ratio(grm, fit, trait, X, vr_geno, order, num_markers, ratio_cv_cutoff, maxiter, tol)[0])
    return out


def loco_grm(grm, geno, begin, end):
    """GRM with GRM markers [begin, end] left out (parallelCrossProd_LOCO FIT.cpp:1790-1851 and
    getDiagOfSigma_LOCO FIT.cpp:2370-2392): (Z'Z - Z_j'Z_j) / (M - M_j), diag minus sum_j z^2."""
    zj = plink.std_geno(geno)[begin:end + 1].astype(np.float64)
    mj = zj.shape[0]
    m = grm.m_qc
    K = (grm.K * m - zj.T @ zj) / (m - mj)
    return DenseGRM.from_matrix(K, m - mj, grm.diag_sum - (zj * zj).sum(axis=0), grm.is_diag_one)


def get_coef_loco(grm_loco, fit0, fit, trait, maxiter_pcg=500, tol_pcg=1e-5, maxiter=20):
    """Get_Coef_LOCO (FIT.R:40-73) from the full fit's tau, alpha and eta (FIT.R:254-297)."""
    fam = Binomial() if trait == "binary" else Gaussian()
    n = len(fit0["y"])
    offset = np.zeros(n) if fit0.get("offset") is None else np.asarray(fit0["offset"], np.float64)
    return get_coef(grm_loco, fit0["y"], fit0["X"], fit["theta"], fam, fit["coefficients"],
                    fit["linear_predictors"], offset, maxiter_pcg, tol_pcg, maxiter)
