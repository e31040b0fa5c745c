"""GLM families used by the null-model fit (R ``binomial(logit)`` and ``gaussian``).

The working vector and weights of ``Get_Coef`` (src/SAIGE/R/SAIGE_fitGLMM_fast.R:2-35)
come from ``linkinv``, ``mu.eta`` and ``variance``; the logit forms follow R's
C_logit_linkinv / C_logit_mu_eta thresholds (|eta| > 30 clamps to DBL_EPSILON).
"""
import numpy as np

_EPS = np.finfo(np.float64).eps


class Binomial:
    name = "binomial"

    def linkinv(self, eta):
        eta = np.asarray(eta, np.float64)
        tmp = np.where(eta < -30.0, _EPS, np.where(eta > 30.0, 1.0 / _EPS, np.exp(np.clip(eta, -30, 30))))
        return tmp / (1.0 + tmp)

    def mu_eta(self, eta):
        eta = np.asarray(eta, np.float64)
        e = np.exp(np.clip(eta, -30, 30))
        return np.where((eta > 30.0) | (eta < -30.0), _EPS, e / ((1.0 + e) * (1.0 + e)))

    def variance(self, mu):
        return mu * (1.0 - mu)

    def parts(self, eta):
        """(linkinv, mu_eta, variance) of eta with one exponential; bit-identical to the
        three separate calls."""
        eta = np.asarray(eta, np.float64)
        e = np.exp(np.clip(eta, -30, 30))
        lo, hi = eta < -30.0, eta > 30.0
        tmp = np.where(lo, _EPS, np.where(hi, 1.0 / _EPS, e))
        mu = tmp / (1.0 + tmp)
        mu_eta = np.where(hi | lo, _EPS, e / ((1.0 + e) * (1.0 + e)))
        return mu, mu_eta, mu * (1.0 - mu)

    def deviance(self, y, mu):
        with np.errstate(divide="ignore", invalid="ignore"):
            a = np.where(y > 0, y * np.log(y / mu), 0.0)
            b = np.where(y < 1, (1 - y) * np.log((1 - y) / (1 - mu)), 0.0)
        return float(2.0 * np.sum(a + b))


class Gaussian:
    name = "gaussian"

    def linkinv(self, eta):
        return np.array(eta, np.float64, copy=True)

    def mu_eta(self, eta):
        return np.ones_like(np.asarray(eta, np.float64))

    def variance(self, mu):
        return np.ones_like(np.asarray(mu, np.float64))

    def parts(self, eta):
        mu = np.array(eta, np.float64, copy=True)
        one = np.ones_like(mu)
        return mu, one, one

    def deviance(self, y, mu):
        return float(np.sum((y - mu) ** 2))


def family_of(name):
    return Binomial() if name in ("binomial", "binary") else Gaussian()
