// Small dense linear algebra on the host (p x p covariate systems of the null-model fit).
#pragma once
#include <algorithm>
#include <cmath>
#include <vector>

namespace sg {

// inverse of a symmetric positive definite matrix (upper triangle used, like
// arma::symmatu) by Cholesky; falls back to the pseudo-inverse from a Jacobi
// eigen-decomposition (arma::pinv) when it is not positive definite.
inline std::vector<double> inv_sympd(const std::vector<double>& A0, int p) {
  std::vector<double> A(p * p);
  for (int i = 0; i < p; ++i)
    for (int j = 0; j < p; ++j) A[i + j * p] = (i <= j) ? A0[i + j * p] : A0[j + i * p];
  std::vector<double> L(p * p, 0.0);
  bool ok = true;
  for (int j = 0; j < p && ok; ++j) {
    double s = A[j + j * p];
    for (int k = 0; k < j; ++k) s -= L[j + k * p] * L[j + k * p];
    if (!(s > 0.0)) { ok = false; break; }
    L[j + j * p] = std::sqrt(s);
    for (int i = j + 1; i < p; ++i) {
      double t = A[i + j * p];
      for (int k = 0; k < j; ++k) t -= L[i + k * p] * L[j + k * p];
      L[i + j * p] = t / L[j + j * p];
    }
  }
  std::vector<double> inv(p * p, 0.0);
  if (ok) {
    std::vector<double> Li(p * p, 0.0);  // L^-1
    for (int j = 0; j < p; ++j) {
      Li[j + j * p] = 1.0 / L[j + j * p];
      for (int i = j + 1; i < p; ++i) {
        double s = 0.0;
        for (int k = j; k < i; ++k) s += L[i + k * p] * Li[k + j * p];
        Li[i + j * p] = -s / L[i + i * p];
      }
    }
    for (int i = 0; i < p; ++i)
      for (int j = 0; j < p; ++j) {
        double s = 0.0;
        for (int k = std::max(i, j); k < p; ++k) s += Li[k + i * p] * Li[k + j * p];
        inv[i + j * p] = s;
      }
    return inv;
  }
  // Jacobi eigen-decomposition, pseudo-inverse with tolerance p * max|lambda| * eps
  std::vector<double> V(p * p, 0.0), D(A);
  for (int i = 0; i < p; ++i) V[i + i * p] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0;
    for (int i = 0; i < p; ++i)
      for (int j = i + 1; j < p; ++j) off += D[i + j * p] * D[i + j * p];
    if (off < 1e-30) break;
    for (int pi = 0; pi < p; ++pi)
      for (int q = pi + 1; q < p; ++q) {
        const double apq = D[pi + q * p];
        if (std::fabs(apq) < 1e-300) continue;
        const double theta = (D[q + q * p] - D[pi + pi * p]) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double cs = 1.0 / std::sqrt(t * t + 1.0), sn = t * cs;
        for (int k = 0; k < p; ++k) {
          const double dkp = D[k + pi * p], dkq = D[k + q * p];
          D[k + pi * p] = cs * dkp - sn * dkq;
          D[k + q * p] = sn * dkp + cs * dkq;
        }
        for (int k = 0; k < p; ++k) {
          const double dpk = D[pi + k * p], dqk = D[q + k * p];
          D[pi + k * p] = cs * dpk - sn * dqk;
          D[q + k * p] = sn * dpk + cs * dqk;
        }
        for (int k = 0; k < p; ++k) {
          const double vkp = V[k + pi * p], vkq = V[k + q * p];
          V[k + pi * p] = cs * vkp - sn * vkq;
          V[k + q * p] = sn * vkp + cs * vkq;
        }
      }
  }
  double mx = 0.0;
  for (int i = 0; i < p; ++i) mx = std::max(mx, std::fabs(D[i + i * p]));
  const double tolv = p * mx * 2.220446049250313e-16;
  for (int i = 0; i < p; ++i)
    for (int j = 0; j < p; ++j) {
      double s = 0.0;
      for (int k = 0; k < p; ++k) {
        const double l = D[k + k * p];
        if (std::fabs(l) > tolv) s += V[i + k * p] * V[j + k * p] / l;
      }
      inv[i + j * p] = s;
    }
  return inv;
}

}  // namespace sg
