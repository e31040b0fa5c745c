/*
 * CPU restatement of the reference's own CPU path for GRM.x and the PCG
 * (TEST / BASELINE INFRASTRUCTURE ONLY -- never linked into libsaigegpu).
 *
 * cpuref_crossprod restates parallelCrossProdOpenMP
 * (src/SAIGE/src/SAIGE_fitGLMM_fast.cpp:1576-1598) and parallelCrossProd's
 * division by M (:1669-1708): for every GRM marker, decode its re-packed
 * 2-bit genotypes through the 3-entry float LUT (Get_OneSNP_StdGeno
 * :582-662), val = dot(z, b) in float, out += val * z, with an OpenMP
 * reduction over markers; then out / M.
 *
 * cpuref_pcg restates getPCG1ofSigmaAndVector (:2593-2809) in float with
 * the Jacobi preconditioner of getDiagOfSigma (:2322-2365) and getCrossprod
 * (:2397-2425).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

static inline int field_geno(unsigned f) { return 2 - (int)((f & 1u) + (f >> 1)); }

void cpuref_crossprod(const uint8_t* packed, int64_t pitch, const float* lut4, int64_t m_qc,
                      int64_t n, const float* b, float* out, int nthreads) {
  if (nthreads > 0) omp_set_num_threads(nthreads);
  int nt = 1;
#pragma omp parallel
  {
#pragma omp single
    nt = omp_get_num_threads();
  }
  float* acc = (float*)calloc((size_t)nt * (size_t)n, sizeof(float));
  float* zbuf = (float*)malloc((size_t)nt * (size_t)n * sizeof(float));
#pragma omp parallel
  {
    const int t = omp_get_thread_num();
    float* a = acc + (size_t)t * n;
    float* z = zbuf + (size_t)t * n;
#pragma omp for schedule(static)
    for (int64_t m = 0; m < m_qc; ++m) {
      const uint8_t* row = packed + m * pitch;
      const float* lut = lut4 + 4 * m;
      float val = 0.0f;
      for (int64_t i = 0; i < n; ++i) {
        z[i] = lut[field_geno((row[i >> 2] >> (2 * (i & 3))) & 3u)];
        val += z[i] * b[i];
      }
      for (int64_t i = 0; i < n; ++i) a[i] += val * z[i];
    }
  }
  const float M = (float)m_qc;
  for (int64_t i = 0; i < n; ++i) {
    float s = 0.0f;
    for (int t = 0; t < nt; ++t) s += acc[(size_t)t * n + i];
    out[i] = s / M;
  }
  free(acc);
  free(zbuf);
}

static float dotf(const float* a, const float* b, int64_t n) {
  float s = 0.0f;
  for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

int cpuref_pcg(const uint8_t* packed, int64_t pitch, const float* lut4, int64_t m_qc, int64_t n,
               const float* diag32, const float* w, const float* tau, const float* b, int maxiter,
               float tol, float* x, int nthreads) {
  float* r = (float*)malloc(n * sizeof(float));
  float* z = (float*)malloc(n * sizeof(float));
  float* p = (float*)malloc(n * sizeof(float));
  float* ap = (float*)malloc(n * sizeof(float));
  float* kp = (float*)malloc(n * sizeof(float));
  float* minv = (float*)malloc(n * sizeof(float));
  const float M = (float)m_qc;
  for (int64_t i = 0; i < n; ++i) {
    float d = (tau[1] * diag32[i]) / M + tau[0] / w[i];
    if (d < 1e-4f) d = 1e-4f;
    minv[i] = 1.0f / d;
    x[i] = 0.0f;
    r[i] = b[i];
    z[i] = minv[i] * r[i];
    p[i] = z[i];
  }
  float sumr2 = dotf(r, r, n);
  int iter = 0;
  while (sumr2 > tol && iter < maxiter) {
    ++iter;
    if (tau[1] != 0.0f) cpuref_crossprod(packed, pitch, lut4, m_qc, n, p, kp, nthreads);
    for (int64_t i = 0; i < n; ++i)
      ap[i] = tau[0] * (p[i] * (1.0f / w[i])) + (tau[1] != 0.0f ? tau[1] * kp[i] : 0.0f);
    const float rz = dotf(r, z, n);
    const float a = rz / dotf(p, ap, n);
    for (int64_t i = 0; i < n; ++i) {
      x[i] += a * p[i];
      r[i] -= a * ap[i];
    }
    for (int64_t i = 0; i < n; ++i) z[i] = minv[i] * r[i];
    const float bet = dotf(z, r, n) / rz;
    for (int64_t i = 0; i < n; ++i) p[i] = z[i] + bet * p[i];
    sumr2 = dotf(r, r, n);
  }
  free(r); free(z); free(p); free(ap); free(kp); free(minv);
  return iter;
}
