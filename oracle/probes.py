"""Counter-based hash used for Hutchinson probes and synthetic cohorts.

The reference draws its probes with R's ``rbinom`` after
``pbdMPI::comm.set.seed(200)`` (FIT.cpp:3040-3054, GetTrace :3135-3137).
R's RNG cannot be reproduced outside R, so this build replaces it with a
stateless counter hash that the CUDA kernels evaluate identically: probe
entry ``u[run, i]`` depends only on ``(seed, run, i)``, so any batching of
probes gives the same vectors.

Hash: three rounds of the splitmix64 finaliser (Steele, Lea & Flood,
"Fast splittable pseudorandom number generators", OOPSLA 2014), keyed as

    h = mix(seed ^ K0);  h = mix(h ^ (stream * K1));  h = mix(h ^ (idx * K2))

with all arithmetic mod 2**64.  A probe entry is +1 when the top bit of
``h`` is set, else -1 (the reference's ``2*rbinom(n,1,0.5)-1``).
"""
import numpy as np

K0 = np.uint64(0x5851F42D4C957F2D)
K1 = np.uint64(0x9E3779B97F4A7C15)
K2 = np.uint64(0xD1B54A32D192ED03)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def mix64(z):
    z = np.asarray(z, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


def hash3(seed, stream, idx):
    """Vectorised hash of (seed, stream, idx) -> uint64 (broadcasts)."""
    seed = np.asarray(seed, dtype=np.uint64)
    stream = np.asarray(stream, dtype=np.uint64)
    idx = np.asarray(idx, dtype=np.uint64)
    with np.errstate(over="ignore"):
        h = mix64(seed ^ K0)
        h = mix64(h ^ (stream * K1))
        h = mix64(h ^ (idx * K2))
    return h


def rademacher(seed, run, n, index=None):
    """Probe vector u (length n, float64 in {-1,+1}) for probe number ``run``.

    ``index``: the sample numbers the hash takes (default 0..n-1).  A phenotype whose samples are a
    subset S of a cohort hashes the cohort positions S, as the engine masks the cohort's probes."""
    idx = np.arange(n, dtype=np.uint64) if index is None else np.asarray(index, dtype=np.uint64)
    h = hash3(seed, np.uint64(run), idx)
    return np.where((h >> np.uint64(63)) == 1, 1.0, -1.0)


def rademacher_block(seed, run0, nrun, n):
    """Probes run0 .. run0+nrun-1 as an (nrun, n) array."""
    return np.stack([rademacher(seed, run0 + k, n) for k in range(nrun)])
