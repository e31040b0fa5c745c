"""Host-side phenotype preparation that precedes the null-model fit.

Mirrors the R code of ``fitNULLGLMM`` that builds ``fit0`` before
``glmmkin.ai_PCG_Rcpp_*`` is called (src/SAIGE/R/SAIGE_fitGLMM_fast.R):

* ``covariate_transform``: ``Covariate_Transform`` (FIT.R:1612-1648) -- QR of
  the design, columns ``Q * sqrt(N)``;
* ``glm_fit``: R's ``glm`` IRLS for ``binomial(logit)`` / ``gaussian(identity)``
  (FIT.R:1119-1129) with R's starting values and deviance test;
* ``make_fit0``: the ``isCovariateOffset`` branch (FIT.R:1108-1117, 1126-1129),
  which turns the covariate part of the linear predictor into an offset and
  refits an intercept-only model.

This is host logic, not the GPU hot path; it runs once per phenotype.
"""
import numpy as np

from .family import Binomial, Gaussian


def covariate_transform(X):
    """Covariate_Transform (FIT.R:1612-1648): Q * sqrt(N) of the design ``X`` (with intercept).

    Collinear columns (NA coefficients in R's ``lm``) are dropped first.
    Householder QR (LAPACK) gives the same signs as R's LINPACK ``qr`` for the
    leading intercept column (R[0,0] = -sqrt(N)).
    """
    X = np.asarray(X, np.float64)
    q, r = np.linalg.qr(X)
    keep = np.abs(np.diag(r)) > 1e-7 * max(1.0, np.abs(np.diag(r)).max())
    if not keep.all():
        X = X[:, keep]
        q, r = np.linalg.qr(X)
    n = X.shape[0]
    return q * np.sqrt(n), r, keep


def glm_fit(y, X, family, offset=None, maxit=25, epsilon=1e-8):
    """R ``glm.fit`` IRLS (weights 1). Returns coefficients, linear predictors, fitted values."""
    y = np.asarray(y, np.float64)
    X = np.asarray(X, np.float64)
    n = len(y)
    off = np.zeros(n) if offset is None else np.asarray(offset, np.float64)
    if family.name == "binomial":
        mustart = (y + 0.5) / 2.0
        eta = np.log(mustart / (1.0 - mustart))
    else:
        eta = y.copy()
    mu = family.linkinv(eta)
    dev_old = family.deviance(y, mu)
    beta = np.zeros(X.shape[1])
    for _ in range(maxit):
        mu_eta = family.mu_eta(eta)
        z = (eta - off) + (y - mu) / mu_eta
        w = np.sqrt(mu_eta ** 2 / family.variance(mu))
        beta, *_ = np.linalg.lstsq(X * w[:, None], z * w, rcond=None)
        eta = X @ beta + off
        mu = family.linkinv(eta)
        dev = family.deviance(y, mu)
        if abs(dev - dev_old) / (abs(dev) + 0.1) < epsilon:
            break
        dev_old = dev
    return dict(coefficients=beta, linear_predictors=eta, fitted_values=mu)


def make_fit0(y, covariates, trait="binary", covariate_offset=True, covariate_transform_qr=True):
    """Build ``fit0`` as fitNULLGLMM does (FIT.R:1040-1129) for the null-model fit.

    ``covariates`` is (n, q) without the intercept (q may be 0).  Returns a
    dict with y, X, offset, linear_predictors, coefficients and family name, and
    with the QR transform its R factor and kept columns (``transform``), which
    Covariate_Transform_Back (FIT.R:1653-1659) needs.
    """
    y = np.asarray(y, np.float64)
    n = len(y)
    family = Binomial() if trait == "binary" else Gaussian()
    C = np.zeros((n, 0)) if covariates is None else np.asarray(covariates, np.float64).reshape(n, -1)
    has_cov = C.shape[1] > 0
    X = np.column_stack([np.ones(n), C])
    if not has_cov:
        covariate_offset = False
    transform = None
    if covariate_transform_qr and has_cov:
        X, qrr, keep = covariate_transform(X)
        transform = dict(qrr=qrr, keep=keep)
    g = glm_fit(y, X, family)
    if covariate_offset:
        covoffset = X[:, 1:] @ g["coefficients"][1:]
        X0 = np.ones((n, 1))
        g0 = glm_fit(y, X0, family, offset=covoffset)
        return dict(y=y, X=X0, offset=covoffset, linear_predictors=g0["linear_predictors"],
                    coefficients=g0["coefficients"], family=family.name, Xorig=X, transform=transform)
    return dict(y=y, X=X, offset=None, linear_predictors=g["linear_predictors"],
                coefficients=g["coefficients"], family=family.name, Xorig=None, transform=transform)
