"""Seeded synthetic cohorts with the shapes of the benchmark configurations.

Genotypes follow the integer recipe that ``sg_synth_bed`` evaluates on the GPU
(csrc/k_geno.cu), so small cohorts made here on the CPU are byte-identical to
the device-made ones:

* marker m: ``thr_m = 167772 + (((hash3(seed,1,m) >> 40) * 8220835) >> 24)`` --
  allele frequency p_m = thr_m / 2^24 in [0.01, 0.5);
* sample i: ``h = hash3(seed, 16+m, i)``; two allele draws
  ``(h >> 40) < thr_m`` and ``((h >> 16) & 0xFFFFFF) < thr_m`` (HWE);
  missing when ``(h & 0xFFFF) < round(miss_rate * 65536)``;
* PLINK SNP-major coding of the counted allele: 2 -> 00, 1 -> 10, 0 -> 11,
  missing -> 01, with the 3-byte magic 6C 1B 01.

Phenotypes: a polygenic value g = sqrt(tau) * Z b / sqrt(M) (b ~ N(0,1)),
standard-normal covariates, then a logistic (binary, intercept solved for the
target prevalence) or linear (quantitative, target heritability) model.
"""
import numpy as np

_K0 = np.uint64(0x5851F42D4C957F2D)
_K1 = np.uint64(0x9E3779B97F4A7C15)
_K2 = np.uint64(0xD1B54A32D192ED03)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def _mix(z):
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


def hash3(seed, stream, idx):
    seed = np.asarray(seed, np.uint64)
    stream = np.asarray(stream, np.uint64)
    idx = np.asarray(idx, np.uint64)
    with np.errstate(over="ignore"):
        h = _mix(seed ^ _K0)
        h = _mix(h ^ (stream * _K1))
        return _mix(h ^ (idx * _K2))


def marker_thresholds(seed, m):
    hm = hash3(seed, 1, np.arange(m, dtype=np.uint64))
    return (np.uint64(167772) + (((hm >> np.uint64(40)) * np.uint64(8220835)) >> np.uint64(24))).astype(np.uint64)


def synth_bed(seed, n, m, miss_rate):
    """(bytes of a .bed, genotype codes (m, n) with 3 = missing)."""
    thr = marker_thresholds(seed, m)
    miss_thr = np.uint64(int(round(miss_rate * 65536.0)))
    idx = np.arange(n, dtype=np.uint64)
    nb = (n + 3) // 4
    body = np.zeros((m, nb), np.uint8)
    codes = np.zeros((m, n), np.uint8)
    for j in range(m):
        h = hash3(seed, 16 + j, idx)
        a1 = (h >> np.uint64(40)) < thr[j]
        a2 = ((h >> np.uint64(16)) & np.uint64(0xFFFFFF)) < thr[j]
        g = a1.astype(np.uint8) + a2.astype(np.uint8)
        miss = (h & np.uint64(0xFFFF)) < miss_thr
        field = np.where(g == 2, 0, np.where(g == 1, 2, 3)).astype(np.uint8)
        field[miss] = 1
        codes[j] = np.where(miss, 3, g)
        f = np.zeros(nb * 4, np.uint8)
        f[:n] = field
        f = f.reshape(nb, 4)
        body[j] = f[:, 0] | (f[:, 1] << 2) | (f[:, 2] << 4) | (f[:, 3] << 6)
    return bytes([0x6C, 0x1B, 0x01]) + body.tobytes(), codes


def standard_normal(seed, stream, n):
    """Box-Muller normals from the counter hash (float64)."""
    i = np.arange(n, dtype=np.uint64)
    u1 = ((hash3(seed, stream, i) >> np.uint64(11)).astype(np.float64) + 0.5) * 2.0 ** -53
    u2 = (hash3(seed, stream + 1, i) >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)


def genetic_value_from_codes(codes, seed):
    """g = Z b / sqrt(M) with Z standardised on the observed (non-missing) frequencies."""
    m, n = codes.shape
    b = standard_normal(seed, 2, m)
    acc = np.zeros(n)
    for j in range(m):
        c = codes[j].astype(np.float64)
        ok = codes[j] != 3
        p = c[ok].mean() / 2.0 if ok.any() else 0.0
        sd = np.sqrt(2 * p * (1 - p))
        if sd == 0:
            continue
        z = np.where(ok, (c - 2 * p) / sd, 0.0)
        acc += z * b[j]
    return acc / np.sqrt(m)


def simulate_pheno(g, seed, trait="binary", tau=0.3, prevalence=0.2, h2=0.4, n_cov=2):
    """Phenotype from a genetic value g (variance ~1): returns (y, covariates (n, n_cov))."""
    n = len(g)
    X = np.column_stack([standard_normal(seed, 100 + 2 * k, n) for k in range(n_cov)]) if n_cov else np.zeros((n, 0))
    if trait == "binary":
        lin = X.sum(axis=1) * 0.5 + np.sqrt(tau) * g
        # intercept for the target prevalence (bisection on the mean of the logistic)
        lo, hi = -20.0, 20.0
        for _ in range(80):
            mid = 0.5 * (lo + hi)
            if np.mean(1.0 / (1.0 + np.exp(-(mid + lin)))) > prevalence:
                hi = mid
            else:
                lo = mid
        prob = 1.0 / (1.0 + np.exp(-(0.5 * (lo + hi) + lin)))
        u = (hash3(seed, 200, np.arange(n, dtype=np.uint64)) >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
        y = (u < prob).astype(np.float64)
    else:
        e = standard_normal(seed, 300, n)
        y = X.sum(axis=1) * 0.3 + np.sqrt(h2) * g + np.sqrt(1 - h2) * e
    return y, X
