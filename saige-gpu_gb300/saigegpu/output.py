"""Step-1 outputs in the layout step 2 reads (FIT.R:1297-1301, 2416-2417).

Without R the ``.rda`` model cannot be written; ``write_model`` writes the same
``modglmm`` fields (theta, coefficients, linear.predictors, fitted.values, Y,
residuals, cov, converged, traitType, sampleID) as a JSON sidecar that an R
maintainer can turn into the list with ``jsonlite::fromJSON``.  The variance
ratio file is the reference's plain text table: value, "null", category.
"""
import json

import numpy as np


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
