// Multi-RHS Jacobi-PCG engine kernels (FP64 vectors and recurrences).
//
// Each column c runs the loop of getPCG1ofSigmaAndVector
// (src/SAIGE/src/SAIGE_fitGLMM_fast.cpp:2593-2809) on its own:
//     x = 0, r = b, z = M^-1 r, p = z
//     while (r'r > tol && iter < maxiter):
//         Ap = tau0 p / W + tau1 K p                      (getCrossprod :2397-2425)
//         a = r'z / p'Ap;  x += a p;  r1 = r - a Ap;  z1 = M^-1 r1
//         b = z1'r1 / z'r; p = z1 + b p;  iter++
// The GRM product K p of all in-flight columns is one GEMM per engine step;
// the kernels below are the FP64 vector work around it, split at the two
// reductions.  Reductions are two-level and in a fixed order (block partials,
// then a sequential sum per column), so a column's arithmetic does not depend
// on how many other columns share the step.
//
// Vectors are RHS-major: column c occupies [c*np, (c+1)*np).  A phenotype
// slot g contributes winv = 1/W and minv = 1/diag(Sigma) rows, both 0 outside
// the phenotype's sample subset (which keeps the subset's columns exact).
#include "sg_internal.h"

namespace sg {

constexpr int kThreads = 256;
constexpr int kChunk = 2048;  // vector elements per block
// The vector kernels move two consecutive elements per thread and iteration (16-byte FP64 and
// 8-byte FP32 accesses; np is even, so every column starts 16-byte aligned), four iterations per
// block, unrolled so that their loads are in flight together.
constexpr int kVecIters = kChunk / (2 * kThreads);

__device__ __forceinline__ double2 ld2(const double* p) { return *reinterpret_cast<const double2*>(p); }
__device__ __forceinline__ void st2(double* p, double a, double b) {
  *reinterpret_cast<double2*>(p) = make_double2(a, b);
}
__device__ __forceinline__ void st2f(float* p, float a, float b) {
  *reinterpret_cast<float2*>(p) = make_float2(a, b);
}
__device__ __forceinline__ double2 ld2y(const float* Yf, const double* Yd, int64_t i) {
  if (Yf) {
    const float2 v = *reinterpret_cast<const float2*>(Yf + i);
    return make_double2((double)v.x, (double)v.y);
  }
  return ld2(Yd + i);
}

int64_t pcg_nblk(int64_t np) { return (np + kChunk - 1) / kChunk; }

__device__ __forceinline__ double block_sum(double v, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0) {
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh[i];
  }
  __syncthreads();
  return s;
}

// Admit columns cols[0..n): x = 0, r = mask*b, z = minv r, p = z; partial r'z, r'r.
// Product columns (kind 1) only stage Pf = mask*b.
__global__ void pcg_init_kernel(int64_t np, const int32_t* __restrict__ cols,
                                const ColState* __restrict__ st, const double* __restrict__ minv,
                                const double* __restrict__ B, double* X, double* R, double* Z,
                                double* P, float* Pf, double* part, int64_t nblk) {
  __shared__ double sh[kThreads / 32];
  const int sel = blockIdx.y;
  const int64_t c = cols[sel];
  const ColState s = st[c];
  const double* mv = minv + (int64_t)s.pheno * np;
  const double* b = B + (int64_t)sel * np;
  const int64_t base = c * np;
  const int64_t i0 = (int64_t)blockIdx.x * kChunk;
  double zr = 0.0, rr = 0.0;
#pragma unroll
  for (int it = 0; it < kVecIters; ++it) {
    const int64_t i = i0 + 2 * (it * kThreads + threadIdx.x);
    if (i >= np) break;
    const double2 m = ld2(mv + i), bb = ld2(b + i);
    const double b0 = (m.x != 0.0) ? bb.x : 0.0, b1 = (m.y != 0.0) ? bb.y : 0.0;
    st2(X + base + i, 0.0, 0.0);
    if (s.kind == 0) {
      const double z0 = m.x * b0, z1 = m.y * b1;
      st2(R + base + i, b0, b1);
      st2(Z + base + i, z0, z1);
      st2(P + base + i, z0, z1);
      st2f(Pf + base + i, (float)z0, (float)z1);
      zr += z0 * b0;
      zr += z1 * b1;
      rr += b0 * b0;
      rr += b1 * b1;
    } else {
      st2f(Pf + base + i, (float)b0, (float)b1);
    }
  }
  zr = block_sum(zr, sh);
  rr = block_sum(rr, sh);
  if (threadIdx.x == 0) {
    part[(c * nblk + blockIdx.x) * 2 + 0] = zr;
    part[(c * nblk + blockIdx.x) * 2 + 1] = rr;
  }
}

__global__ void pcg_init_finalize_kernel(const int32_t* __restrict__ cols, int64_t ncols_sel,
                                         ColState* st, const double* __restrict__ part,
                                         int64_t nblk) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= ncols_sel) return;
  const int64_t c = cols[k];
  ColState s = st[c];
  double zr = 0.0, rr = 0.0;
  for (int64_t b = 0; b < nblk; ++b) {
    zr += part[(c * nblk + b) * 2 + 0];
    rr += part[(c * nblk + b) * 2 + 1];
  }
  s.iter = 0;
  s.just_done = 0;
  s.alpha = 0.0;
  s.beta = 0.0;
  if (s.kind == 0) {
    s.rz = zr;
    s.r2 = rr;
    s.active = (rr > s.tol && s.maxiter > 0) ? 1 : 0;
    if (!s.active) s.just_done = 1;
  } else {
    s.active = 1;
  }
  st[c] = s;
}

void launch_pcg_init(int64_t np, int64_t ncols, const int32_t* cols, int64_t ncols_sel,
                     ColState* st, const PhenoState* ph, const double* minv, const double* B,
                     double* X, double* R, double* Z, double* P, float* Pf, double* part,
                     int64_t nblk, cudaStream_t s) {
  (void)ncols; (void)ph;
  if (ncols_sel == 0) return;
  dim3 grid((unsigned)nblk, (unsigned)ncols_sel);
  pcg_init_kernel<<<grid, kThreads, 0, s>>>(np, cols, st, minv, B, X, R, Z, P, Pf, part, nblk);
  pcg_init_finalize_kernel<<<(unsigned)((ncols_sel + 127) / 128), 128, 0, s>>>(cols, ncols_sel, st,
                                                                               part, nblk);
}

__device__ __forceinline__ double ap_value(double tau0, double tau1, double winv, double m,
                                           double p, double y) {
  return (m != 0.0) ? (tau0 * winv * p + tau1 * y) : 0.0;
}

// partial p'Ap for active PCG columns
__global__ void pcg_sigma_dot_kernel(int64_t np, const ColState* __restrict__ st,
                                     const PhenoState* __restrict__ ph,
                                     const double* __restrict__ winv, const double* __restrict__ minv,
                                     const double* __restrict__ P, const float* __restrict__ Yf,
                                     const double* __restrict__ Yd, double* part, int64_t nblk,
                                     const int32_t* __restrict__ cols) {
  __shared__ double sh[kThreads / 32];
  const int64_t c = cols ? cols[blockIdx.y] : blockIdx.y;
  const ColState s = st[c];
  if (s.kind != 0 || !s.active) {
    if (threadIdx.x == 0) part[(c * nblk + blockIdx.x) * 2] = 0.0;
    return;
  }
  const PhenoState g = ph[s.pheno];
  const double* wv = winv + (int64_t)s.pheno * np;
  const double* mv = minv + (int64_t)s.pheno * np;
  const int64_t base = c * np;
  const int64_t i0 = (int64_t)blockIdx.x * kChunk;
  double acc = 0.0;
#pragma unroll
  for (int it = 0; it < kVecIters; ++it) {
    const int64_t i = i0 + 2 * (it * kThreads + threadIdx.x);
    if (i >= np) break;
    const double2 p = ld2(P + base + i), y = ld2y(Yf, Yd, base + i), w = ld2(wv + i), m = ld2(mv + i);
    acc += p.x * ap_value(g.tau0, g.tau1, w.x, m.x, p.x, y.x);
    acc += p.y * ap_value(g.tau0, g.tau1, w.y, m.y, p.y, y.y);
  }
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) part[(c * nblk + blockIdx.x) * 2] = acc;
}

void launch_pcg_sigma_dot(int64_t np, int64_t ncols, ColState* st, const PhenoState* ph,
                          const double* winv, const double* minv, const double* P,
                          const float* Yf, const double* Yd, double* part, int64_t nblk,
                          const int32_t* cols, cudaStream_t s) {
  if (ncols == 0) return;
  dim3 grid((unsigned)nblk, (unsigned)ncols);
  pcg_sigma_dot_kernel<<<grid, kThreads, 0, s>>>(np, st, ph, winv, minv, P, Yf, Yd, part, nblk, cols);
}

__global__ void pcg_alpha_kernel(int64_t ncols, ColState* st, const double* __restrict__ part,
                                 int64_t nblk, const int32_t* __restrict__ cols) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= ncols) return;
  const int64_t c = cols ? cols[j] : j;
  ColState s = st[c];
  if (s.kind != 0 || !s.active) {
    s.alpha = 0.0;
  } else {
    double pap = 0.0;
    for (int64_t b = 0; b < nblk; ++b) pap += part[(c * nblk + b) * 2];
    s.alpha = s.rz / pap;
  }
  st[c].alpha = s.alpha;
}

void launch_pcg_alpha(int64_t ncols, ColState* st, const double* part, int64_t nblk,
                      const int32_t* cols, cudaStream_t s) {
  if (ncols == 0) return;
  pcg_alpha_kernel<<<(unsigned)((ncols + 127) / 128), 128, 0, s>>>(ncols, st, part, nblk, cols);
}

// x += a p; r -= a Ap; z = minv r; partial z'r, r'r.  Product columns copy K b into X.
__global__ void pcg_update_kernel(int64_t np, const ColState* __restrict__ st,
                                  const PhenoState* __restrict__ ph, const double* __restrict__ winv,
                                  const double* __restrict__ minv, double* X, double* R, double* Z,
                                  const double* __restrict__ P, const float* __restrict__ Yf,
                                  const double* __restrict__ Yd, double* part, int64_t nblk,
                                  const int32_t* __restrict__ cols) {
  __shared__ double sh[kThreads / 32];
  const int64_t c = cols ? cols[blockIdx.y] : blockIdx.y;
  const ColState s = st[c];
  const int64_t base = c * np;
  const int64_t i0 = (int64_t)blockIdx.x * kChunk;
  if (!s.active) {
    if (threadIdx.x == 0) {
      part[(c * nblk + blockIdx.x) * 2 + 0] = 0.0;
      part[(c * nblk + blockIdx.x) * 2 + 1] = 0.0;
    }
    return;
  }
  const double* mv = minv + (int64_t)s.pheno * np;
  if (s.kind == 1) {
#pragma unroll
    for (int it = 0; it < kVecIters; ++it) {
      const int64_t i = i0 + 2 * (it * kThreads + threadIdx.x);
      if (i >= np) break;
      const double2 y = ld2y(Yf, Yd, base + i), m = ld2(mv + i);
      st2(X + base + i, (m.x != 0.0) ? y.x : 0.0, (m.y != 0.0) ? y.y : 0.0);
    }
    return;
  }
  const PhenoState g = ph[s.pheno];
  const double* wv = winv + (int64_t)s.pheno * np;
  const double a = s.alpha;
  double zr = 0.0, rr = 0.0;
#pragma unroll
  for (int it = 0; it < kVecIters; ++it) {
    const int64_t i = i0 + 2 * (it * kThreads + threadIdx.x);
    if (i >= np) break;
    const double2 p = ld2(P + base + i), y = ld2y(Yf, Yd, base + i), m = ld2(mv + i), w = ld2(wv + i);
    const double2 x = ld2(X + base + i), r0 = ld2(R + base + i);
    const double ap0 = ap_value(g.tau0, g.tau1, w.x, m.x, p.x, y.x);
    const double ap1 = ap_value(g.tau0, g.tau1, w.y, m.y, p.y, y.y);
    st2(X + base + i, x.x + a * p.x, x.y + a * p.y);
    const double ra = r0.x - a * ap0, rb = r0.y - a * ap1;
    const double za = m.x * ra, zb = m.y * rb;
    st2(R + base + i, ra, rb);
    st2(Z + base + i, za, zb);
    zr += za * ra;
    zr += zb * rb;
    rr += ra * ra;
    rr += rb * rb;
  }
  zr = block_sum(zr, sh);
  rr = block_sum(rr, sh);
  if (threadIdx.x == 0) {
    part[(c * nblk + blockIdx.x) * 2 + 0] = zr;
    part[(c * nblk + blockIdx.x) * 2 + 1] = rr;
  }
}

void launch_pcg_update(int64_t np, int64_t ncols, ColState* st, const PhenoState* ph,
                       const double* winv, const double* minv, double* X, double* R, double* Z,
                       const double* P, const float* Yf, const double* Yd, double* part,
                       int64_t nblk, const int32_t* cols, cudaStream_t s) {
  if (ncols == 0) return;
  dim3 grid((unsigned)nblk, (unsigned)ncols);
  pcg_update_kernel<<<grid, kThreads, 0, s>>>(np, st, ph, winv, minv, X, R, Z, P, Yf, Yd, part, nblk, cols);
}

// beta, iteration count and the stopping rule (sum r^2 <= tol or iter == maxiter)
__global__ void pcg_beta_kernel(int64_t ncols, ColState* st, const double* __restrict__ part,
                                int64_t nblk, const int32_t* __restrict__ cols) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= ncols) return;
  const int64_t c = cols ? cols[j] : j;
  ColState s = st[c];
  s.just_done = 0;
  if (s.active) {
    if (s.kind == 1) {
      s.active = 0;
      s.just_done = 1;
      s.iter = 1;
    } else {
      double zr = 0.0, rr = 0.0;
      for (int64_t b = 0; b < nblk; ++b) {
        zr += part[(c * nblk + b) * 2 + 0];
        rr += part[(c * nblk + b) * 2 + 1];
      }
      s.beta = zr / s.rz;
      s.rz = zr;
      s.r2 = rr;
      s.iter += 1;
      if (!(rr > s.tol && s.iter < s.maxiter)) {
        s.active = 0;
        s.just_done = 1;
      }
    }
  }
  st[c] = s;
}

void launch_pcg_beta(int64_t ncols, ColState* st, const double* part, int64_t nblk,
                     const int32_t* cols, cudaStream_t s) {
  if (ncols == 0) return;
  pcg_beta_kernel<<<(unsigned)((ncols + 127) / 128), 128, 0, s>>>(ncols, st, part, nblk, cols);
}

// p = z + beta p for columns still iterating; FP32 copy for the next GRM product.
__global__ void pcg_dir_kernel(int64_t np, const ColState* __restrict__ st, const double* __restrict__ Z,
                               double* P, float* Pf, const int32_t* __restrict__ cols) {
  const int64_t c = cols ? cols[blockIdx.y] : blockIdx.y;
  const ColState s = st[c];
  const int64_t base = c * np;
  const int64_t i0 = (int64_t)blockIdx.x * kChunk;
  if (s.active && s.kind == 0) {
    const double b = s.beta;
#pragma unroll
    for (int it = 0; it < kVecIters; ++it) {
      const int64_t i = i0 + 2 * (it * kThreads + threadIdx.x);
      if (i >= np) break;
      const double2 z = ld2(Z + base + i), p = ld2(P + base + i);
      const double pa = z.x + b * p.x, pb = z.y + b * p.y;
      st2(P + base + i, pa, pb);
      st2f(Pf + base + i, (float)pa, (float)pb);
    }
  } else if (s.just_done) {
#pragma unroll
    for (int it = 0; it < kVecIters; ++it) {
      const int64_t i = i0 + 2 * (it * kThreads + threadIdx.x);
      if (i >= np) break;
      st2f(Pf + base + i, 0.0f, 0.0f);
    }
  }
}

void launch_pcg_dir(int64_t np, int64_t ncols, ColState* st, const double* Z, double* P, float* Pf,
                    const int32_t* cols, cudaStream_t s) {
  if (ncols == 0) return;
  dim3 grid((unsigned)pcg_nblk(np), (unsigned)ncols);
  pcg_dir_kernel<<<grid, kThreads, 0, s>>>(np, st, Z, P, Pf, cols);
}

// Rademacher probes of the counter hash (oracle/probes.py): B[j][i] = +-1 for i < nn, 0 after.
__global__ void probe_fill_kernel(int64_t np, int64_t nn, uint64_t seed, int64_t run0,
                                  double* B) {
  const int64_t j = blockIdx.y;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  double v = 0.0;
  if (i < nn) v = (hash3(seed, (uint64_t)(run0 + j), (uint64_t)i) >> 63) ? 1.0 : -1.0;
  B[j * np + i] = v;
}

void launch_probe_fill(int64_t np, int64_t nn, uint64_t seed, int64_t run0, int64_t k, double* B,
                       cudaStream_t s) {
  if (k == 0) return;
  dim3 grid((unsigned)((np + 255) / 256), (unsigned)k);
  probe_fill_kernel<<<grid, 256, 0, s>>>(np, nn, seed, run0, B);
}

// Probes for a set of staging rows in one launch: row sel[j] of B gets probe (seeds[j], runs[j]).
__global__ void probe_fill_multi_kernel(int64_t np, int64_t nn, const uint64_t* __restrict__ seeds,
                                        const int64_t* __restrict__ runs, const int32_t* __restrict__ sel,
                                        double* B) {
  const int64_t j = blockIdx.y;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  double v = 0.0;
  if (i < nn) v = (hash3(seeds[j], (uint64_t)runs[j], (uint64_t)i) >> 63) ? 1.0 : -1.0;
  B[(int64_t)sel[j] * np + i] = v;
}

void launch_probe_fill_multi(int64_t np, int64_t nn, const uint64_t* seeds, const int64_t* runs,
                             const int32_t* sel, int64_t k, double* B, cudaStream_t s) {
  if (k == 0) return;
  dim3 grid((unsigned)((np + 255) / 256), (unsigned)k);
  probe_fill_multi_kernel<<<grid, 256, 0, s>>>(np, nn, seeds, runs, sel, B);
}

// Hutchinson probe reductions: for probe j the block sums of Au.Su, u.Su, Au.SX_q and SX_q.u.
// Blocks of 128 threads with the accumulators sized for p <= 4 (the usual covariate count) take
// few enough registers to run on an SM beside a genotype-GEMM CTA, in its idle issue slots.
constexpr int kDotsThreads = 128;

template <int PMAX>
__global__ void __launch_bounds__(kDotsThreads)
probe_dots_kernel(int64_t np, int64_t nn, const double* const* __restrict__ vecs, int64_t k,
                  const double* __restrict__ minv, uint64_t seed, int64_t run0,
                  const double* __restrict__ SX, int p, double* part, int64_t nblk) {
  __shared__ double sh[kDotsThreads / 32];
  const int64_t j = blockIdx.y;
  const double* su = vecs[j];
  const double* au = vecs[k + j];
  const int64_t i0 = (int64_t)blockIdx.x * kChunk;
  double v[2 + 2 * PMAX];
#pragma unroll
  for (int q = 0; q < 2 + 2 * PMAX; ++q) v[q] = 0.0;
  for (int64_t i = i0 + threadIdx.x; i < i0 + kChunk && i < nn; i += kDotsThreads) {
    const double a = au[i], s = su[i];
    const double u = (minv[i] != 0.0) ? ((hash3(seed, (uint64_t)(run0 + j), (uint64_t)i) >> 63) ? 1.0 : -1.0) : 0.0;
    v[0] += a * s;
    v[1] += u * s;
#pragma unroll
    for (int q = 0; q < PMAX; ++q) {
      if (q < p) {
        const double x = SX[(int64_t)q * np + i];
        v[2 + q] += a * x;
        v[2 + PMAX + q] += x * u;
      }
    }
  }
  const int nv = 2 + 2 * p;
  for (int q = 0; q < nv; ++q) {
    const int src = q < 2 + p ? q : (2 + PMAX + (q - 2 - p));
    const double t = block_sum(v[src], sh);
    if (threadIdx.x == 0) part[(j * nblk + blockIdx.x) * nv + q] = t;
  }
}

void launch_probe_dots(int64_t np, int64_t nn, const double* const* vecs, int64_t k,
                       const double* minv_row, uint64_t seed, int64_t run0, const double* SX,
                       int64_t p, double* part, int64_t nblk, cudaStream_t s) {
  if (k == 0) return;
  dim3 grid((unsigned)nblk, (unsigned)k);
  if (p <= 4)
    probe_dots_kernel<4><<<grid, kDotsThreads, 0, s>>>(np, nn, vecs, k, minv_row, seed, run0, SX, (int)p, part, nblk);
  else
    probe_dots_kernel<kProbeDotsMaxP><<<grid, kDotsThreads, 0, s>>>(np, nn, vecs, k, minv_row, seed, run0, SX, (int)p,
                                                                  part, nblk);
}

__global__ void f64_to_f32_kernel(const double* a, float* b, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}
__global__ void f32_to_f64_kernel(const float* a, double* b, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (double)a[i];
}
void launch_f64_to_f32(const double* a, float* b, int64_t n, cudaStream_t s) {
  if (n) f64_to_f32_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a, b, n);
}
void launch_f32_to_f64(const float* a, double* b, int64_t n, cudaStream_t s) {
  if (n) f32_to_f64_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a, b, n);
}


// A phenotype slot's 1/W and Jacobi preconditioner 1/diag(Sigma) (getDiagOfSigma FIT.cpp:2322-2365:
// tau1 diagK / M + tau0 / W, or tau1 + tau0 / W with isDiagofKinSetAsOne, floored at 1e-4), zero
// outside the sample subset and past nn; IEEE-rounded operations in the reference's order.
__global__ void slot_weights_kernel(int64_t np, int64_t nn, const double* __restrict__ w,
                                    const uint8_t* __restrict__ mask, const double* __restrict__ diag,
                                    double m, double tau0, double tau1, int diag_one,
                                    double* __restrict__ winv, double* __restrict__ minv) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  if (i >= nn || (mask && !mask[i])) {
    winv[i] = 0.0;
    minv[i] = 0.0;
    return;
  }
  const double wi = w[i];
  const double t = __ddiv_rn(tau0, wi);
  const double v = diag_one ? __dadd_rn(tau1, t) : __dadd_rn(__ddiv_rn(__dmul_rn(tau1, diag[i]), m), t);
  winv[i] = __ddiv_rn(1.0, wi);
  minv[i] = __ddiv_rn(1.0, v < 1e-4 ? 1e-4 : v);
}

void launch_slot_weights(int64_t np, int64_t nn, const double* w, const uint8_t* mask, const double* diag,
                         double m, double tau0, double tau1, int diag_one, double* winv, double* minv,
                         cudaStream_t s) {
  slot_weights_kernel<<<(unsigned)((np + 255) / 256), 256, 0, s>>>(np, nn, w, mask, diag, m, tau0, tau1,
                                                                   diag_one, winv, minv);
}

// d_st[cols[k]] = src[k]: column states staged by the host in one block; a column set free
// (kind -1) also gets a zero FP32 direction, so padding columns of a GRM.V pass contribute nothing.
// One block per staged column.
__global__ void scatter_states_kernel(const ColState* __restrict__ src, const int32_t* __restrict__ cols,
                                      int64_t n, ColState* __restrict__ dst, float* __restrict__ Pf, int64_t np) {
  const int64_t k = blockIdx.x;
  if (k >= n) return;
  const ColState st = src[k];
  const int64_t c = cols[k];
  if (threadIdx.x == 0) dst[c] = st;
  if (Pf && st.kind == -1)
    for (int64_t i = threadIdx.x; i < np; i += blockDim.x) Pf[c * np + i] = 0.0f;
}

void launch_scatter_states(const ColState* src, const int32_t* cols, int64_t n, ColState* dst, float* Pf,
                           int64_t np, cudaStream_t s) {
  if (n <= 0) return;
  scatter_states_kernel<<<(unsigned)n, 256, 0, s>>>(src, cols, n, dst, Pf, np);
}

// Right-hand sides of an admission round: column sel[k] of B (np rows) = the nn values at host
// address src[k] (pinned and mapped), zero past nn.  One block per column.
__global__ void gather_rhs_kernel(const double* const* __restrict__ src, const int32_t* __restrict__ sel,
                                  int64_t n, int64_t nn, int64_t np, double* __restrict__ B) {
  const int64_t k = blockIdx.x;
  if (k >= n) return;
  const double* x = src[k];
  double* b = B + (int64_t)sel[k] * np;
  for (int64_t i = threadIdx.x; i < np; i += blockDim.x) b[i] = i < nn ? x[i] : 0.0;
}

void launch_gather_rhs(const double* const* src, const int32_t* sel, int64_t n, int64_t nn, int64_t np, double* B,
                       cudaStream_t s) {
  if (n <= 0) return;
  gather_rhs_kernel<<<(unsigned)n, 256, 0, s>>>(src, sel, n, nn, np, B);
}

}  // namespace sg
