"""Host driver of the null-model fit, mirroring the reference's R functions.

``get_coef`` mirrors ``Get_Coef`` (src/SAIGE/R/SAIGE_fitGLMM_fast.R:2-35),
``glmmkin_binary`` / ``glmmkin_quantitative`` mirror
``glmmkin.ai_PCG_Rcpp_Binary`` (:79-304) and ``_Quantitative`` (:309-549),
without LOCO.  They call the GPU drop-ins of the Rcpp entry points
(``Context.getCoefficients``, ``getAIScore``, ``fitglmmaiRPCG`` ...) exactly
where the R code calls ``.Call``; like Rcpp, the boundary carries float32
vectors and the driver keeps double precision on its side.
"""
import numpy as np

from .family import family_of


def get_coef(ctx, y, X, tau, family, alpha0, eta0, offset, maxiter_pcg, tol_pcg, maxiter):
    """Get_Coef (FIT.R:2-35)."""
    tol_coef = 0.1
    mu = family.linkinv(eta0)
    mu_eta = family.mu_eta(eta0)
    Y = eta0 - offset + (y - mu) / mu_eta
    W = (mu_eta / np.sqrt(family.variance(mu))) ** 2
    for _ in range(maxiter):
        rc = ctx.getCoefficients(Y, X, W, tau, maxiter_pcg, tol_pcg)
        alpha = rc["alpha"].astype(np.float64)
        eta = rc["eta"].astype(np.float64) + offset
        mu = family.linkinv(eta)
        mu_eta = family.mu_eta(eta)
        Y = eta - offset + (y - mu) / mu_eta
        W = (mu_eta / np.sqrt(family.variance(mu))) ** 2
        if np.max(np.abs(alpha - alpha0) / (np.abs(alpha) + np.abs(alpha0) + tol_coef)) < tol_coef:
            break
        alpha0 = alpha
    return dict(Y=Y, alpha=alpha, eta=eta, W=W, cov=rc["cov"], Sigma_iY=rc["Sigma_iY"],
                Sigma_iX=rc["Sigma_iX"], mu=mu)


def _start(fit0):
    y = np.asarray(fit0["y"], np.float64)
    X = np.asarray(fit0["X"], np.float64)
    n = len(y)
    off = fit0.get("offset")
    off = np.zeros(n) if off is None else np.asarray(off, np.float64)
    return y, X, n, off, np.asarray(fit0["linear_predictors"], np.float64), np.asarray(fit0["coefficients"], np.float64)


def glmmkin_binary(ctx, fit0, tol=0.02, maxiter=20, nrun=30, tol_pcg=1e-5, maxiter_pcg=500,
                   trace_cv_cutoff=0.0025, tau_init=(0.0, 0.0), seed=200):
    """glmmkin.ai_PCG_Rcpp_Binary (FIT.R:79-304) on the GPU drop-ins."""
    fam = family_of("binomial")
    y, X, n, offset, eta, alpha0 = _start(fit0)
    eta0 = eta
    tau = np.array([1.0, 0.1 if tau_init[1] == 0 else tau_init[1]])
    tau0 = tau.copy()
    rc = get_coef(ctx, y, X, tau, fam, alpha0, eta0, offset, maxiter_pcg, tol_pcg, maxiter)
    re = ctx.getAIScore(rc["Y"], X, rc["W"], tau, rc["Sigma_iY"], rc["Sigma_iX"], rc["cov"], nrun,
                        maxiter_pcg, tol_pcg, trace_cv_cutoff, seed)
    tau[1] = max(0.0, tau0[1] + tau0[1] ** 2 * (re["YPAPY"] - re["Trace"]) / n)
    it_used = 0
    for i in range(1, maxiter + 1):
        it_used = i
        alpha0 = rc["alpha"]
        tau0 = tau.copy()
        eta0 = eta
        rc = get_coef(ctx, y, X, tau, fam, alpha0, eta0, offset, maxiter_pcg, tol_pcg, maxiter)
        fit = ctx.fitglmmaiRPCG(rc["Y"], X, rc["W"], tau, rc["Sigma_iY"], rc["Sigma_iX"], rc["cov"],
                                nrun, maxiter_pcg, tol_pcg, tol, trace_cv_cutoff, seed)
        tau = fit["tau"].astype(np.float64)
        alpha, eta = rc["alpha"], rc["eta"]
        if tau[1] == 0:
            break
        if np.max(np.abs(tau - tau0) / (np.abs(tau) + np.abs(tau0) + tol)) < tol:
            break
        if np.max(tau) > tol ** (-2):
            it_used = maxiter
            break
    rc = get_coef(ctx, y, X, tau, fam, alpha, eta, offset, maxiter_pcg, tol_pcg, maxiter)
    return dict(theta=tau, coefficients=rc["alpha"], linear_predictors=rc["eta"],
                fitted_values=rc["mu"], Y=rc["Y"], residuals=y - rc["mu"], cov=rc["cov"],
                converged=it_used < maxiter, iterations=it_used)


def glmmkin_quantitative(ctx, fit0, tol=0.02, maxiter=20, nrun=30, tol_pcg=1e-5, maxiter_pcg=500,
                         trace_cv_cutoff=0.0025, tau_init=(0.0, 0.0), seed=200):
    """glmmkin.ai_PCG_Rcpp_Quantitative (FIT.R:309-549) on the GPU drop-ins."""
    fam = family_of("gaussian")
    y, X, n, offset, eta, alpha = _start(fit0)
    Y = eta - offset + (y - fam.linkinv(eta)) / fam.mu_eta(eta)
    alpha0 = alpha
    eta0 = eta
    if sum(tau_init) == 0:
        tau = np.array([1.0, 0.0])
        if abs(np.var(Y, ddof=1)) < 0.1:
            raise ValueError("variance of the phenotype is much smaller than 1")
    else:
        tau = np.array(tau_init, np.float64)
    tau0 = tau.copy()
    rc = get_coef(ctx, y, X, tau, fam, alpha0, eta0, offset, maxiter_pcg, tol_pcg, maxiter)
    re = ctx.getAIScore_q(rc["Y"], X, rc["W"], tau, rc["Sigma_iY"], rc["Sigma_iX"], rc["cov"], nrun,
                          maxiter_pcg, tol_pcg, trace_cv_cutoff, seed)
    tau[1] = max(0.0, tau0[1] + tau0[1] ** 2 * (re["YPAPY"] - re["Trace"][1]) / n)
    tau[0] = max(0.0, tau0[0] + tau0[0] ** 2 * (re["YPA0PY"] - re["Trace"][0]) / n)
    it_used = 0
    for i in range(1, maxiter + 1):
        it_used = i
        alpha0 = alpha
        tau0 = tau.copy()
        eta0 = eta
        rc = get_coef(ctx, y, X, tau, fam, alpha0, eta0, offset, maxiter_pcg, tol_pcg, maxiter)
        fit = ctx.fitglmmaiRPCG(rc["Y"], X, rc["W"], tau, rc["Sigma_iY"], rc["Sigma_iX"], rc["cov"],
                                nrun, maxiter_pcg, tol_pcg, tol, trace_cv_cutoff, seed,
                                quantitative=True)
        tau = fit["tau"].astype(np.float64)
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
    rc = get_coef(ctx, y, X, tau, fam, alpha, eta, offset, maxiter_pcg, tol_pcg, maxiter)
    return dict(theta=tau, coefficients=rc["alpha"], linear_predictors=rc["eta"],
                fitted_values=rc["mu"], Y=rc["Y"], residuals=y - rc["mu"], cov=rc["cov"],
                converged=it_used < maxiter, iterations=it_used)
