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
#include <math.h>
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

/* Same counter hash and synthetic-cohort recipe as the GPU generator (saigegpu/synth.py),
 * followed by the reference's setgeno for the identity sample order (QC, integer fill,
 * float frequency and 1/sd, re-pack; FIT.cpp:326-579, 739-1024).  Writes the re-packed
 * GRM markers (pitch bytes per marker) and their LUTs; returns the number of GRM markers. */
static inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static inline uint64_t hash3(uint64_t seed, uint64_t stream, uint64_t idx) {
  uint64_t h = mix64(seed ^ 0x5851F42D4C957F2Dull);
  h = mix64(h ^ (stream * 0x9E3779B97F4A7C15ull));
  return mix64(h ^ (idx * 0xD1B54A32D192ED03ull));
}

int64_t cpuref_synth_setgeno(uint64_t seed, int64_t n, int64_t m, double miss_rate, float min_maf,
                             float max_miss, uint8_t* packed, int64_t pitch, float* lut4,
                             int nthreads) {
  if (nthreads > 0) omp_set_num_threads(nthreads);
  const uint32_t miss_thr = (uint32_t)(miss_rate * 65536.0 + 0.5);
  int8_t* pass = (int8_t*)calloc((size_t)m, 1);
  float* lut_all = (float*)malloc((size_t)m * 4 * sizeof(float));
  uint8_t* rows = (uint8_t*)malloc((size_t)m * (size_t)pitch);
#pragma omp parallel
  {
    uint8_t* g = (uint8_t*)malloc((size_t)n);
#pragma omp for schedule(dynamic, 64)
    for (int64_t j = 0; j < m; ++j) {
      const uint64_t hm = hash3(seed, 1ull, (uint64_t)j);
      const uint32_t thr = 167772u + (uint32_t)(((hm >> 40) * 8220835ull) >> 24);
      int allele = 0, nmiss = 0;
      for (int64_t i = 0; i < n; ++i) {
        const uint64_t h = hash3(seed, 16ull + (uint64_t)j, (uint64_t)i);
        if ((uint32_t)(h & 0xFFFFu) < miss_thr) { g[i] = 3; ++nmiss; continue; }
        g[i] = (uint8_t)(((uint32_t)(h >> 40) < thr) + ((uint32_t)((h >> 16) & 0xFFFFFFu) < thr));
        allele += g[i];
      }
      const float alt0 = (float)allele / (float)((n - nmiss) * 2);
      const int fill = (alt0 == alt0) ? (int)floor((double)(2.0f * alt0) + 0.5) : 0;
      if (nmiss > 0) allele += fill * nmiss;
      const float alt = (float)allele / (float)(n * 2);
      const float maf = alt < 1.0f - alt ? alt : 1.0f - alt;
      const float mrate = (float)nmiss / (float)n;
      pass[j] = (maf >= min_maf && mrate <= max_miss) ? 1 : 0;
      const float sd = sqrtf(2.0f * alt * (1.0f - alt));
      const float inv = sd == 0.0f ? 0.0f : 1.0f / sd;
      const float p2 = 2.0f * alt;
      lut_all[4 * j + 0] = (0.0f - p2) * inv;
      lut_all[4 * j + 1] = (1.0f - p2) * inv;
      lut_all[4 * j + 2] = (2.0f - p2) * inv;
      lut_all[4 * j + 3] = 0.0f;
      uint8_t* row = rows + (size_t)j * pitch;
      memset(row, 0, (size_t)pitch);
      for (int64_t i = 0; i < n; ++i) {
        int gi = g[i] == 3 ? fill : g[i];
        const unsigned code = gi == 0 ? 3u : (gi == 1 ? 2u : 0u);
        row[i >> 2] |= (uint8_t)(code << (2 * (i & 3)));
      }
    }
    free(g);
  }
  int64_t k = 0;
  for (int64_t j = 0; j < m; ++j) {
    if (!pass[j]) continue;
    memcpy(packed + (size_t)k * pitch, rows + (size_t)j * pitch, (size_t)pitch);
    memcpy(lut4 + 4 * k, lut_all + 4 * j, 4 * sizeof(float));
    ++k;
  }
  free(rows); free(lut_all); free(pass);
  return k;
}
