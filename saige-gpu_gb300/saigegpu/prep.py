"""Host-side phenotype preparation that precedes the null-model fit.

Mirrors the R code of ``fitNULLGLMM`` that builds ``fit0`` before
``glmmkin.ai_PCG_Rcpp_*`` is called (src/SAIGE/R/SAIGE_fitGLMM_fast.R):

* ``covariate_transform``: ``Covariate_Transform`` (FIT.R:1612-1648) -- QR of
  the design, columns ``Q * sqrt(N)``;
* ``glm_fit``: R's ``glm`` IRLS for ``binomial(logit)`` / ``gaussian(identity)``
  (FIT.R:1119-1129) with R's starting values and deviance test;
* ``make_fit0``: the ``isCovariateOffset`` branch (FIT.R:1108-1117, 1126-1129),
  which turns the covariate part of the linear predictor into an offset and
  refits an intercept-only model;
* ``read_phenotypes``: the phenotype-file preamble (FIT.R:855-1010): complete
  cases, categorical covariates as R's treatment-contrast columns, the merge
  with the .fam samples in genotype order, inverse normalisation, the binary
  covariates' minimum-count check, and setgeno's sample arguments.

This is host logic, not the GPU hot path; it runs once per phenotype.
"""
import gzip

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


_NA = {"", "NA", "NaN", "nan", "NAN"}


def _r_number_label(v):
    """How R prints a factor level made from a number (as.character of a double)."""
    return "%d" % v if float(v).is_integer() and abs(v) < 1e15 else "%.15g" % v


def _factor_columns(name, values):
    """R's treatment contrasts of factor(values): one 0/1 column per level after the first, named
    name + level (model.matrix); levels sorted as as.factor sorts them (numerically when every
    value is a number)."""
    try:
        nums = np.array([float(v) for v in values])
        levels = sorted(set(nums.tolist()))
        keys = nums
        labels = [_r_number_label(v) for v in levels]
    except ValueError:
        levels = sorted(set(values))
        keys = np.array(values, dtype=object)
        labels = list(levels)
    cols = [(keys == lv).astype(np.float64) for lv in levels[1:]]
    return cols, [name + lab for lab in labels[1:]]


def read_phenotypes(pheno_file, fam_file, pheno_col, covar_cols=(), qcovar_cols=(), sample_id_col="IID",
                    trait="binary", inv_normalize=False, sample_include=None, sex_col=None, female_only=False,
                    male_only=False, female_code="1", male_code="0", min_covariate_count=-1):
    """fitNULLGLMM's phenotype preamble (FIT.R:855-1010) for one phenotype.

    Reads the whitespace-delimited phenotype file (header; .gz allowed), keeps the rows complete in
    the phenotype, covariates and sample ID, optionally only the IDs in ``sample_include`` and one
    sex, builds the design columns of ``pheno ~ covariates`` (``qcovar_cols`` as factors: treatment
    contrasts named as R's model.matrix names them), keeps the samples of the .fam in genotype order
    (merge on IID, ordered by .fam position), inverse-normalises a quantitative phenotype
    (qnorm((rank - 0.5) / n), ties averaged) and, for a binary trait, drops two-valued covariate
    columns with a cell of fewer than ``min_covariate_count`` samples (checkPerfectSep).

    Returns a dict: y, covariates (n x q, without the intercept), covariate_names, sample_ids,
    sub_1based (.fam positions, 1-based, for setgeno's subSampleInGeno) and pheno_mask (.fam-length
    bools, its indicatorGenoSamplesWithPheno), n_fam."""
    from scipy.stats import norm, rankdata
    opener = gzip.open if str(pheno_file).endswith((".gz", ".bgz")) else open
    with opener(pheno_file, "rt") as f:
        rows = [line.split() for line in f if line.strip()]
    header, rows = rows[0], rows[1:]
    covar_cols, qcovar_cols = list(covar_cols), list(qcovar_cols)
    for c in [pheno_col, sample_id_col] + covar_cols + ([sex_col] if (female_only or male_only) else []):
        if c not in header:
            raise ValueError("column %s does not exist in the phenotype file" % c)
    if not set(qcovar_cols) <= set(covar_cols):
        raise ValueError("every categorical covariate must be in the covariate list")
    col = {h: i for i, h in enumerate(header)}
    keep_cols = [pheno_col] + covar_cols + [sample_id_col]
    rows = [r for r in rows if all(r[col[c]] not in _NA for c in keep_cols)]
    if sample_include is not None:
        inc = set(str(s) for s in sample_include)
        rows = [r for r in rows if r[col[sample_id_col]] in inc]
    if female_only or male_only:
        code = female_code if female_only else male_code
        rows = [r for r in rows if r[col[sex_col]] == code]
        if not rows:
            raise ValueError("no samples coded %s in column %s" % (code, sex_col))
    # the genotype samples: .fam IIDs in file order
    fam_ids = [line.split()[1] for line in open(fam_file) if line.strip()]
    pos = {s: k for k, s in enumerate(fam_ids)}
    rows = sorted((r for r in rows if r[col[sample_id_col]] in pos), key=lambda r: pos[r[col[sample_id_col]]])
    if not rows:
        raise ValueError("no sample of the phenotype file is in the .fam")
    ids = [r[col[sample_id_col]] for r in rows]
    y = np.array([float(r[col[pheno_col]]) for r in rows])
    cols, names = [], []
    for c in covar_cols:
        vals = [r[col[c]] for r in rows]
        if c in qcovar_cols:
            fc, fn = _factor_columns(c, vals)
            cols += fc
            names += fn
        else:
            cols.append(np.array([float(v) for v in vals]))
            names.append(c)
    if trait == "quantitative" and inv_normalize:
        y = norm.ppf((rankdata(y) - 0.5) / len(y))
    if trait == "binary":
        if not set(np.unique(y).tolist()) <= {0.0, 1.0}:
            raise ValueError("a binary phenotype takes the values 0 and 1")
        keep = []
        for c, name in zip(cols, names):
            vals = np.unique(c)
            if len(vals) == 2 and min_covariate_count > 0:
                counts = [np.count_nonzero((y == a) & (c == b)) for a in (0.0, 1.0) for b in vals]
                if min(counts) < min_covariate_count:
                    continue
            keep.append((c, name))
        cols, names = [c for c, _ in keep], [n for _, n in keep]
    sub = np.array([pos[s] + 1 for s in ids], dtype=np.int32)
    mask = np.zeros(len(fam_ids), bool)
    mask[sub - 1] = True
    C = np.column_stack(cols) if cols else np.zeros((len(y), 0))
    return dict(y=y, covariates=C, covariate_names=names, sample_ids=ids, sub_1based=sub, pheno_mask=mask,
                n_fam=len(fam_ids))
