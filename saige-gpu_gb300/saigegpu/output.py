"""Step-1 outputs in the layout step 2 reads (FIT.R:1297-1301, 2416-2417).

``write_model_rda`` writes the model as the reference's step 1 saves it: an .rda file (R's own
serialisation, ``saigegpu.rdata``) holding one list ``modglmm`` with the fields, order, shapes and
classes of FIT.R's result lists (FIT.R:239-242 / 495-498, the LOCO results of FIT.R:291 / 536, then
FIT.R:1150-1195), so that step 2's ``load()`` finds what it reads.  ``write_model`` writes the
main fields as a JSON sidecar.  The variance ratio file is the reference's plain text table: value,
"null", category.
"""
import json

import numpy as np

from . import rdata


def write_variance_ratio(path, ratios_by_category):
    """One line per category: '<ratio> null <k>' (write.table of FIT.R:2416-2417)."""
    with open(path, "w") as f:
        for k, r in enumerate(ratios_by_category, start=1):
            f.write("%.14g null %d\n" % (float(r), k))


def read_variance_ratio(path):
    out = []
    for line in open(path):
        parts = line.split()
        if len(parts) >= 2 and parts[1] == "null":
            out.append(float(parts[0]))
    return out


def write_model(path, fit, trait, sample_ids=None, isCovariateOffset=True):
    def arr(v):
        return np.asarray(v, np.float64).ravel().tolist()
    d = {"theta": arr(fit["theta"]), "coefficients": arr(fit["coefficients"]),
         "linear.predictors": arr(fit["linear_predictors"]), "fitted.values": arr(fit["fitted_values"]),
         "Y": arr(fit["Y"]), "residuals": arr(fit["residuals"]), "cov": arr(fit["cov"]),
         "converged": bool(fit["converged"]), "traitType": trait, "isCovariateOffset": bool(isCovariateOffset),
         "LOCO": False}
    if sample_ids is not None:
        d["sampleID"] = [str(s) for s in sample_ids]
    with open(path, "w") as f:
        json.dump(d, f)


def read_model(path):
    d = json.load(open(path))
    for k in ("theta", "coefficients", "linear.predictors", "fitted.values", "Y", "residuals", "cov"):
        d[k] = np.asarray(d[k])
    return d


# ---------------------------------------------------------------------------------- .rda model
def score_test_null_model(mu, mu2, y, X):
    """ScoreTest_NULL_Model (FIT.R:579-591): the no-K score-test pieces, as arrays."""
    V = np.asarray(mu2, np.float64)
    X = np.asarray(X, np.float64)
    res = np.asarray(y, np.float64) - np.asarray(mu, np.float64)
    XV = (X * V[:, None]).T
    XVX = X.T @ XV.T
    XVX_inv = np.linalg.solve(XVX, np.eye(XVX.shape[0]))
    XXVX_inv = X @ XVX_inv
    return dict(XV=XV, XVX=XVX, XXVX_inv=XXVX_inv, XVX_inv=XVX_inv, S_a=(X * res[:, None]).sum(axis=0),
                XVX_inv_XV=XXVX_inv * V[:, None], V=V)


def covariate_transform_back(coef, transform, n):
    """Covariate_Transform_Back (FIT.R:1653-1659): coefficients on the original covariate scale."""
    c = np.asarray(coef, np.float64).reshape(-1) * np.sqrt(n)
    return np.linalg.solve(transform["qrr"], c)


def _noK_object(nk, colnames):
    cn = rdata.r_str(colnames)

    def mat(a, rows_named_by_cols, cols_named):
        a = np.asarray(a, np.float64)
        dn = rdata.r_list([cn if rows_named_by_cols else None, cn if cols_named else None])
        return rdata.RObj(rdata.REALSXP, a.ravel(order="F"),
                          [("dim", rdata.r_int(list(a.shape))), ("dimnames", dn)])
    return rdata.r_named_list([
        ("XV", mat(nk["XV"], True, False)),
        ("XVX", mat(nk["XVX"], True, True)),
        ("XXVX_inv", mat(nk["XXVX_inv"], False, True)),
        ("XVX_inv", mat(nk["XVX_inv"], True, True)),
        ("S_a", rdata.r_double(nk["S_a"], names=colnames)),
        ("XVX_inv_XV", mat(nk["XVX_inv_XV"], False, True)),
        ("V", rdata.r_double(nk["V"])),
    ], cls="SA_NULL")


def _col(v):
    a = np.asarray(v, np.float64).reshape(-1)
    return rdata.r_double(a, dim=(len(a), 1))


def model_object(fit, fit0, trait, sample_ids, covariate_names=None, loco=None, use_sparse_grm=False):
    """The step-1 model ``modglmm`` as an R list (``saigegpu.rdata``).

    fit: a null fit (theta, coefficients, linear_predictors, fitted_values, Y, residuals, cov,
    converged) over the phenotype's samples; fit0: its ``prep.make_fit0``; sample_ids: those
    samples' IIDs; covariate_names: the design's covariate columns without the intercept (named
    "minus1" after Covariate_Transform, else "(Intercept)"); loco: ``serve.fit_loco``'s results for this phenotype,
    {chromosome: dict or None}, or None without LOCO.  Fields as FIT.R assembles them: the fit list
    (239-242 / 495-498), LOCO and LOCOResult (251-295 / 504-540; alpha0 and, without the covariate
    offset, the offset of 1169-1170 on each chromosome), obj.glm.null (1154), offset (1158-1178),
    useSparseGRMtoFitNULL (1195); with the QR transform and no covariate offset the coefficients
    are transformed back (1201-1203).  Row names of y and X (R's data-frame row numbers) are not
    written."""
    quant = trait != "binary"
    y = np.asarray(fit0["y"], np.float64)
    n = len(y)
    offset_mode = fit0.get("offset") is not None
    Xfit = np.asarray(fit0["X"], np.float64)
    Xs = np.asarray(fit0["Xorig"], np.float64) if offset_mode else Xfit  # the X the model keeps
    q = Xs.shape[1] - 1
    cov_names = ["x%d" % (k + 1) for k in range(q)] if covariate_names is None else list(covariate_names)
    if len(cov_names) != q:
        raise ValueError("%d covariate names for %d covariates" % (len(cov_names), q))
    # Covariate_Transform renames the intercept "minus1" (FIT.R:1630-1632); without it R's model
    # matrix calls it "(Intercept)"
    colnames = ["minus1" if fit0.get("transform") is not None else "(Intercept)"] + cov_names
    tau = np.asarray(fit["theta"], np.float64)

    def mu2_of(mu):
        return np.full(n, 1.0 / tau[0]) if quant else mu * (1.0 - mu)

    def coef_object(alpha):
        alpha = np.asarray(alpha, np.float64).reshape(-1)
        if fit0.get("transform") is not None and not offset_mode:
            # solve(qrr, coef) keeps qrr's column names as row names, then names() are X_name
            back = covariate_transform_back(alpha, fit0["transform"], n)
            o = rdata.r_double(back, dim=(len(back), 1))
            o.attrs.append(("dimnames", rdata.r_list([rdata.r_str(["(Intercept)"] + cov_names), None])))
            o.attrs.append(("names", rdata.r_str(colnames)))
            return o
        return rdata.r_double(alpha, dim=(len(alpha), 1))

    def cov_object(c):
        c = np.atleast_2d(np.asarray(c, np.float64))
        return rdata.r_double(c, dim=c.shape)

    mu = np.asarray(fit["fitted_values"], np.float64).reshape(-1)
    nk = score_test_null_model(mu, mu2_of(mu), y, Xs)
    fields = [
        ("theta", rdata.r_double(tau)),
        ("coefficients", coef_object(fit["coefficients"])),
        ("linear.predictors", _col(fit["linear_predictors"])),
        ("fitted.values", _col(mu)),
        ("Y", _col(fit["Y"])),
        ("residuals", _col(y - mu)),
        ("cov", cov_object(fit["cov"])),
        ("converged", rdata.r_lgl(bool(fit.get("converged", True)))),
        ("sampleID", rdata.r_str([str(s) for s in sample_ids])),
        ("obj.noK", _noK_object(nk, colnames)),
        ("y", rdata.r_double(y)),
        ("X", rdata.r_matrix(Xs, colnames)),
        ("traitType", rdata.r_str("quantitative" if quant else "binary")),
        ("isCovariateOffset", rdata.r_lgl(offset_mode)),
        ("LOCO", rdata.r_lgl(loco is not None)),
    ]
    if loco is not None:
        entries = []
        for j in range(1, 23):
            r = loco.get(j)
            if not r or not r.get("isLOCO", False):
                entries.append(rdata.r_named_list([("isLOCO", rdata.r_lgl(False))]))
                continue
            mu_j = np.asarray(r["fitted_values"], np.float64).reshape(-1)
            nk_j = score_test_null_model(mu_j, mu2_of(mu_j), y, Xs)
            alpha = np.asarray(r["coefficients"], np.float64).reshape(-1)
            e = [("isLOCO", rdata.r_lgl(True)), ("coefficients", coef_object(alpha)),
                 ("linear.predictors", _col(r["linear_predictors"])), ("fitted.values", _col(mu_j)),
                 ("Y", _col(r["Y"])), ("residuals", _col(y - mu_j)), ("cov", cov_object(r["cov"])),
                 ("obj.noK", _noK_object(nk_j, colnames)), ("alpha0", _col(alpha))]
            if not offset_mode and Xfit.shape[1] > 1:
                e.append(("offset", _col(Xfit[:, 1:] @ alpha[1:])))
            entries.append(rdata.r_named_list(e))
        lr = rdata.r_list(entries)
        lr.levels = 32  # R grows the list by [[j]] <- ..., which marks it growable
        fields.append(("LOCOResult", lr))
    model = rdata.RObj(rdata.VECSXP, [], [("names", rdata.r_str([])), ("class", rdata.r_str("data.frame")),
                                            ("row.names", rdata.r_int([]))])
    fields.append(("obj.glm.null", rdata.r_named_list([("model", model)])))
    if offset_mode:
        off = np.asarray(fit0["offset"], np.float64)
    elif Xfit.shape[1] > 1:
        off = Xfit[:, 1:] @ np.asarray(fit["coefficients"], np.float64).reshape(-1)[1:]
    else:
        off = np.zeros(n)
    fields.append(("offset", _col(off)))
    fields.append(("useSparseGRMtoFitNULL", rdata.r_lgl(use_sparse_grm)))
    return rdata.r_named_list(fields)


def write_model_rda(path, fit, fit0, trait, sample_ids, covariate_names=None, loco=None, use_sparse_grm=False):
    """save(modglmm, file = path) (FIT.R:1218, 1299)."""
    rdata.write_rda(path, [("modglmm", model_object(fit, fit0, trait, sample_ids, covariate_names, loco,
                                                    use_sparse_grm))])


def read_model_rda(path):
    """The ``modglmm`` list of a step-1 .rda (this package's or the reference's) as a dict: numeric
    fields as numpy arrays in their R shape, character fields as lists, nested lists as dicts,
    LOCOResult as a list of dicts."""
    _, objs = rdata.read_rda(path)
    model = dict(objs).get("modglmm")
    if model is None:
        raise ValueError("no modglmm in %s" % path)

    def conv(x):
        if x is None or isinstance(x, rdata.RAltrep):
            return None
        if x.type in (rdata.LGLSXP, rdata.INTSXP, rdata.REALSXP):
            return rdata.to_numpy(x)
        if x.type == rdata.STRSXP:
            return list(x.value)
        if x.type == rdata.VECSXP:
            names = x.names()
            if names is None:
                return [conv(e) for e in x.value]
            return {k: conv(e) for k, e in zip(names, x.value)}
        return x
    return conv(model)


def write_step1(prefix, fit, fit0, trait, sample_ids, covariate_names=None, loco=None, variance_ratios=None):
    """Step 1's outputs under the reference's outputPrefix convention (FIT.R:1218, 1299, 2416-2417):
    ``<prefix>.rda`` (the model) and, given the ratios (one per MAC category),
    ``<prefix>.varianceRatio.txt``.  Returns the paths written."""
    paths = [str(prefix) + ".rda"]
    write_model_rda(paths[0], fit, fit0, trait, sample_ids, covariate_names, loco)
    if variance_ratios is not None:
        paths.append(str(prefix) + ".varianceRatio.txt")
        write_variance_ratio(paths[1], list(np.atleast_1d(variance_ratios)))
    return paths
