"""How much would an FP64 iterative-refinement outer loop save over the two-product solves?

The subset-exact engine applies K with two BF16 products per GEMM: the vector operand as BF16 high
+ low halves (16 significant bits). The alternative is one product on the high half alone (8
significant bits, half the tensor work), inside an outer loop that computes the residual with the
16-bit operator and solves for the correction with the 8-bit one. This study emulates both on the
host. K is built in FP64 from synthetic genotypes, and only the vector operand is rounded, as on
the GPU, where G is exact in BF16.

Costs are counted in two-product applications of K: a one-product application counts one half.
The direct solve is the reference's Jacobi PCG with its absolute stopping rule
(getPCG1ofSigmaAndVector, FIT.cpp:2593-2809: sum r^2 < tol). The refined solve stops on the same
rule for the outer residual, and each inner solve reduces its residual by ``inner_reduction``.

    python -m saigegpu.refinement_study [--n 2000] [--m 5000]
"""
import argparse
import json

import numpy as np


def bf16(x):
    """Round to BF16 (nearest, ties to even), returned as float64."""
    b = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def split16(v):
    h = bf16(v)
    return h + bf16(v - h)


def _pcg(apply, diag, b, tol, maxiter, x0=None, rel=None):
    """Jacobi PCG; stops on sum r^2 < tol (absolute) or, with rel, on sum r^2 < rel^2 sum b^2.
    Returns (x, iterations)."""
    x = np.zeros_like(b) if x0 is None else x0.copy()
    r = b - apply(x) if x0 is not None else b.copy()
    stop = tol if rel is None else rel * rel * float(b @ b)
    z = r / diag
    p = z.copy()
    rz = float(r @ z)
    it = 0
    while float(r @ r) >= stop and it < maxiter:
        q = apply(p)
        a = rz / float(p @ q)
        x += a * p
        r -= a * q
        z = r / diag
        rz1 = float(r @ z)
        p = z + (rz1 / rz) * p
        rz = rz1
        it += 1
    return x, it


def _grm(codes):
    """K = Z'Z / M over the markers with MAF >= 0.01, missing calls at the mean (a study's K; the
    reference's exact QC and fill rules do not matter for the iteration counts)."""
    g = codes.astype(np.float64)
    miss = codes == 3
    g[miss] = np.nan
    p = np.nanmean(g, axis=1) / 2.0
    keep = np.minimum(p, 1.0 - p) >= 0.01
    g, p = g[keep], p[keep]
    g = np.where(np.isnan(g), 2.0 * p[:, None], g)
    z = (g - 2.0 * p[:, None]) / np.sqrt(2.0 * p * (1.0 - p))[:, None]
    return z.T @ z / z.shape[0]


def study(n=2000, m=5000, seed=7, tol=1e-5, inner_reduction=1e-2, trials=6):
    from . import synth
    _, codes = synth.synth_bed(seed, n, m, 0.01)
    K = _grm(codes)
    rng = np.random.default_rng(seed)
    out = []
    for trait, tau in (("binary", (1.0, 0.3)), ("quantitative", (0.6, 0.4))):
        W = rng.uniform(0.05, 0.25, n) if trait == "binary" else np.ones(n)
        diag = tau[0] / W + tau[1] * np.diag(K)
        sig = lambda v, op: tau[0] * v / W + tau[1] * (K @ op(v))
        s16 = lambda v: sig(v, split16)
        s8 = lambda v: sig(v, bf16)
        rows = []
        for t in range(trials):
            b = rng.choice([-1.0, 1.0], n) if t % 2 else rng.standard_normal(n)
            exact = np.linalg.solve(np.diag(tau[0] / W) + tau[1] * K, b)
            x16, n16 = _pcg(s16, diag, b, tol, 5000)
            # refinement: residual with the 16-bit operator, corrections with the 8-bit one
            x = np.zeros(n)
            outer = inner = 0
            r = b.copy()
            while float(r @ r) >= tol and outer < 50:
                d, k = _pcg(s8, diag, r, tol, 5000, rel=inner_reduction)
                inner += k
                x += d
                r = b - s16(x)
                outer += 1
            err16 = float(np.abs(x16 - exact).max() / np.abs(exact).max())
            err_ref = float(np.abs(x - exact).max() / np.abs(exact).max())
            rows.append(dict(direct_iterations=n16, outer=outer, inner_iterations=inner,
                             cost_direct=float(n16), cost_refined=outer + 0.5 * inner,
                             err_direct=err16, err_refined=err_ref))
        cost_d = float(np.mean([r_["cost_direct"] for r_ in rows]))
        cost_r = float(np.mean([r_["cost_refined"] for r_ in rows]))
        out.append(dict(trait=trait, tau=list(tau), n=n, m=m, tol=tol, inner_reduction=inner_reduction,
                        mean_cost_direct=round(cost_d, 1), mean_cost_refined=round(cost_r, 1),
                        refined_over_direct=round(cost_r / cost_d, 3), solves=rows))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=2000)
    ap.add_argument("--m", type=int, default=5000)
    ap.add_argument("--inner-reduction", type=float, default=1e-2)
    a = ap.parse_args()
    for res in study(a.n, a.m, inner_reduction=a.inner_reduction):
        solves = res.pop("solves")
        print(json.dumps(res))
        for s in solves:
            print("   ", json.dumps(s))


if __name__ == "__main__":
    main()
