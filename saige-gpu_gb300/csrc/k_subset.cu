// Subset-exact GRM.V: K_S v for a phenotype whose sample subset S has its own allele frequencies.
//
// The reference rebuilds the genotype object for every phenotype's samples (setgeno over
// subSampleInGeno / indicatorGenoSamplesWithPheno, src/SAIGE/src/SAIGE_fitGLMM_fast.cpp:376-385,
// 436-495 -- "FIT.cpp" below): allele frequency p', integer fill round(2 p'_nonmissing), QC and
// 1/sd' are those of S, so K_S = Z'_S Z'_S^T / M' with z'_im = (g'_im - 2p'_m) / sd'_m is not the
// cohort GRM restricted to S.  This engine applies K_S without forming it, through the cohort's
// genotype values G (0/1/2, the cohort fill in missing calls), stored twice in BF16 (exact):
//
//   v_c = v - mean_S(v)                 (K_S 1_S = 0, so centring changes nothing but rounding)
//   T   = G^T v_c                       (GEMM 1, marker-major G, two BF16 products of v_c's halves)
//   T  += dF^T v_c                      (missing calls of markers whose subset fill differs)
//   T'  = d' .* T,  d'_m = 1/sd'_m^2 for S's GRM markers, 0 otherwise
//   U   = G T'                          (GEMM 2, sample-major G, two BF16 products of T''s halves)
//   K_S v = (U + dF T' - (2p')^T T') / M'   on S
//
// Every kernel below reduces in a fixed order, so a column's product does not depend on which
// other columns share the step.
#include "sg_internal.h"
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_fp8.h>

namespace sg {

namespace {

constexpr int kThreads = 256;
constexpr int kChunk = 2048;  // vector elements per block of the column reductions

__device__ __forceinline__ int field_geno(uint32_t f) { return 2 - (int)((f & 1u) + (f >> 1)); }

__device__ __forceinline__ double block_sum(double v, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh[i];
  __syncthreads();
  return s;
}

__device__ __forceinline__ float block_max(float v, float* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  float s = 0.0f;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s = fmaxf(s, sh[i]);
  __syncthreads();
  return s;
}

// FP16-high / E4M3-low halves.  A column is multiplied by a power of two that brings its largest
// magnitude (bounded by ``bound``) into [2^14, 2^15): FP16 keeps 11 significant bits of it without
// overflow, and the low half (at most 8 in magnitude) sits in E4M3's normal range for every entry
// within 2^-10 of the largest.  The scale is exact, and is divided out after the GEMM.
__device__ __forceinline__ float pow2_scale(float bound) {
  if (!(bound > 0.0f) || !(bound < 3.0e38f)) return 1.0f;
  int e = 0;
  frexpf(bound, &e);  // bound = f 2^e, f in [0.5, 1)
  return ldexpf(1.0f, min(15 - e, 100));
}
__device__ __forceinline__ void split_f8(float x, __half& h, uint8_t& l) {
  h = __float2half_rn(x);
  l = (uint8_t)__nv_cvt_float_to_fp8(x - __half2float(h), __NV_SATFINITE, __NV_E4M3);
}
__device__ __forceinline__ float e4m3_value(uint8_t l) {
  return __half2float(__half(__nv_cvt_fp8_to_halfraw((__nv_fp8_storage_t)l, __NV_E4M3)));
}
// h + l is exact in FP32 (at most 15 significant bits)
__device__ __forceinline__ float join_f8(__half h, uint8_t l) { return __half2float(h) + e4m3_value(l); }

}  // namespace

// ----------------------------------------------------------------------------------- set-up
// Genotype value g (0, 1, 2) as the bit pattern of each operand type (exact in all of them).
__device__ __forceinline__ uint16_t g_bf16(int g) { return g == 0 ? 0x0000u : g == 1 ? 0x3F80u : 0x4000u; }
__device__ __forceinline__ uint16_t g_f16(int g) { return g == 0 ? 0x0000u : g == 1 ? 0x3C00u : 0x4000u; }
__device__ __forceinline__ uint8_t g_e4m3(int g) { return g == 0 ? 0x00u : g == 1 ? 0x38u : 0x40u; }

// G in both layouts from the cohort's packed codes (missing calls kept as 01): block = 64 markers x
// 128 samples staged through shared memory, written coalesced along samples (marker-major G_mm,
// mg x np) and along markers (sample-major G_sm, np x mg).  Missing calls take the cohort fill;
// rows and columns past m and nn are zero.
// form 0: BF16 G in both layouts (Gmm16, Gsm16 hold BF16 bits); form 1: FP16 G in both layouts and
// E4M3 G in both layouts (Gmm8, Gsm8), for the FP16-high / E4M3-low products.
__global__ void gbuild_kernel(const uint8_t* __restrict__ codes, int64_t pitch, const int32_t* __restrict__ fill,
                              int64_t m, int64_t nn, int64_t mg, int64_t np, int form, uint16_t* __restrict__ Gmm16,
                              uint16_t* __restrict__ Gsm16, uint8_t* __restrict__ Gmm8, uint8_t* __restrict__ Gsm8) {
  __shared__ uint8_t sval[64][128 + 2];
  const int64_t m0 = (int64_t)blockIdx.x * 64;
  const int64_t s0 = (int64_t)blockIdx.y * 128;
  const int tid = threadIdx.x;
  for (int e = tid; e < 64 * 128; e += blockDim.x) {
    const int mm = e >> 7, s = e & 127;
    const int64_t mk = m0 + mm, smp = s0 + s;
    uint8_t g = 0;
    if (mk < m && smp < nn) {
      const uint32_t f = (codes[mk * pitch + (smp >> 2)] >> (2 * (smp & 3))) & 3u;
      g = (uint8_t)(f == 1u ? fill[mk] : field_geno(f));
    }
    sval[mm][s] = g;
    Gmm16[mk * np + smp] = form ? g_f16(g) : g_bf16(g);
    if (form) Gmm8[mk * np + smp] = g_e4m3(g);
  }
  __syncthreads();
  for (int e = tid; e < 64 * 128; e += blockDim.x) {
    const int mm = e & 63, s = e >> 6;
    const int g = sval[mm][s];
    Gsm16[(s0 + s) * mg + m0 + mm] = form ? g_f16(g) : g_bf16(g);
    if (form) Gsm8[(s0 + s) * mg + m0 + mm] = g_e4m3(g);
  }
}

void launch_gbuild(const uint8_t* codes, int64_t pitch, const int32_t* fill, int64_t m, int64_t nn,
                   int64_t mg, int64_t np, int form, void* Gmm16, void* Gsm16, void* Gmm8, void* Gsm8,
                   cudaStream_t s) {
  dim3 grid((unsigned)(mg / 64), (unsigned)(np / 128));
  gbuild_kernel<<<grid, kThreads, 0, s>>>(codes, pitch, fill, m, nn, mg, np, form, static_cast<uint16_t*>(Gmm16),
                                          static_cast<uint16_t*>(Gsm16), static_cast<uint8_t*>(Gmm8),
                                          static_cast<uint8_t*>(Gsm8));
}

// A subset's GRM tables from its per-marker QC records, as setgeno over the subset builds them
// (the LUT's 2p and 1/sd: FIT.cpp:152-159): for each GRM marker of the subset, d' = (1/sd')^2,
// 2p', and lut4 = d' (g - 2p')^2 for the four packed codes (00 -> 2, 01 -> the subset's own fill,
// 10 -> 1, 11 -> 0); zeros elsewhere and past m.  flag bit 0: a GRM marker whose subset fill
// differs from the cohort fill G holds; bit 1: a GRM marker of the subset.  Markers ex_lo..ex_hi
// (one chromosome left out; none when ex_lo > ex_hi) are not GRM markers of the subset: the
// subset's GRM over the remaining markers is K_-j of setStartEndIndex + parallelCrossProd_LOCO
// (FIT.cpp:3067-3085, 1790-1851), its diagonal that of set_Diagof_StdGeno_LOCO (FIT.cpp:4934-4959).
__global__ void subset_derive_kernel(const MarkerQC* __restrict__ qc, const int32_t* __restrict__ fill_all,
                                     int64_t m, int64_t mg, int64_t ex_lo, int64_t ex_hi, float* __restrict__ dp,
                                     float* __restrict__ p2, float4* __restrict__ lut4, uint8_t* __restrict__ flag) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= mg) return;
  float d32 = 0.0f, tp = 0.0f;
  float4 l = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  uint8_t f = 0;
  if (k < m && (k < ex_lo || k > ex_hi)) {
    const MarkerQC q = qc[k];
    if (q.pass_qc) {
      const double d = (double)q.invstd * (double)q.invstd;
      const float two_p = 2.0f * q.freq;
      d32 = (float)d;
      tp = two_p;
      const double t0 = 2.0 - (double)two_p, t1 = (double)q.fill - (double)two_p;
      const double t2 = 1.0 - (double)two_p, t3 = 0.0 - (double)two_p;
      l.x = (float)(d * t0 * t0);
      l.y = (float)(d * t1 * t1);
      l.z = (float)(d * t2 * t2);
      l.w = (float)(d * t3 * t3);
      f = (uint8_t)(2u | (q.fill != fill_all[k] ? 1u : 0u));
    }
  }
  dp[k] = d32;
  p2[k] = tp;
  lut4[k] = l;
  flag[k] = f;
}

// The fill-changed markers in marker order (flips, and dfill = subset fill - cohort fill) and the
// counts (nflip, M') in counts[0..1]: one block, each thread a contiguous run of markers, an
// exclusive scan of the runs' flip counts giving each run its output offset.
constexpr int kFlipThreads = 1024;

__global__ void __launch_bounds__(kFlipThreads)
subset_flips_kernel(const MarkerQC* __restrict__ qc, const int32_t* __restrict__ fill_all,
                    const uint8_t* __restrict__ flag, int64_t m, int32_t* __restrict__ flips,
                    float* __restrict__ dfill, int64_t* __restrict__ counts) {
  __shared__ int32_t scan[kFlipThreads];
  __shared__ int32_t grm[kFlipThreads];
  const int t = threadIdx.x;
  const int64_t per = (m + kFlipThreads - 1) / kFlipThreads;
  const int64_t k0 = (int64_t)t * per;
  const int64_t k1 = k0 + per < m ? k0 + per : m;
  int32_t nf = 0, ng = 0;
  for (int64_t k = k0; k < k1; ++k) {
    const uint8_t f = flag[k];
    nf += f & 1u;
    ng += (f >> 1) & 1u;
  }
  scan[t] = nf;
  grm[t] = ng;
  __syncthreads();
  // inclusive Hillis-Steele scan of the flip counts, tree sum of the GRM-marker counts
  for (int o = 1; o < kFlipThreads; o <<= 1) {
    const int32_t a = t >= o ? scan[t - o] : 0;
    __syncthreads();
    scan[t] += a;
    __syncthreads();
  }
  for (int o = kFlipThreads / 2; o > 0; o >>= 1) {
    if (t < o) grm[t] += grm[t + o];
    __syncthreads();
  }
  int32_t pos = scan[t] - nf;
  for (int64_t k = k0; k < k1; ++k)
    if (flag[k] & 1u) {
      flips[pos] = (int32_t)k;
      dfill[pos] = (float)(qc[k].fill - fill_all[k]);
      ++pos;
    }
  if (t == 0) {
    counts[0] = scan[kFlipThreads - 1];
    counts[1] = grm[0];
  }
}

void launch_subset_derive(const MarkerQC* qc, const int32_t* fill_all, int64_t m, int64_t mg, int64_t ex_lo,
                          int64_t ex_hi, float* dp, float* p2, float* lut4, uint8_t* flag, int32_t* flips, float* dfill,
                          int64_t* counts, cudaStream_t s) {
  subset_derive_kernel<<<(unsigned)((mg + kThreads - 1) / kThreads), kThreads, 0, s>>>(
      qc, fill_all, m, mg, ex_lo, ex_hi, dp, p2, reinterpret_cast<float4*>(lut4), flag);
  subset_flips_kernel<<<1, kFlipThreads, 0, s>>>(qc, fill_all, flag, m, flips, dfill, counts);
}

// Bit map of a slot's fill-changed markers, word-major (word w of sample i at bits[w * np + i], so
// that a warp's samples read consecutive words): bit b is set when marker flips[32 w + b] is
// missing at sample i and i is in the subset (mask).
__global__ void subset_bitmap_kernel(const uint8_t* __restrict__ codes, int64_t pitch,
                                     const int32_t* __restrict__ flips, int nflip, int W,
                                     const uint8_t* __restrict__ mask, int64_t nn, int64_t np,
                                     uint32_t* __restrict__ bits) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int w = blockIdx.y;
  if (i >= np) return;
  uint32_t word = 0;
  if (i < nn && (!mask || mask[i])) {
    for (int b = 0; b < 32; ++b) {
      const int k = 32 * w + b;
      if (k >= nflip) break;
      const int64_t mk = flips[k];
      const uint32_t f = (codes[mk * pitch + (i >> 2)] >> (2 * (i & 3))) & 3u;
      if (f == 1u) word |= 1u << b;
    }
  }
  bits[(int64_t)w * np + i] = word;
}

void launch_subset_bitmap(const uint8_t* codes, int64_t pitch, const int32_t* flips, int nflip, int W,
                          const uint8_t* mask, int64_t nn, int64_t np, uint32_t* bits, cudaStream_t s) {
  if (W == 0) return;
  dim3 grid((unsigned)((np + kThreads - 1) / kThreads), (unsigned)W);
  subset_bitmap_kernel<<<grid, kThreads, 0, s>>>(codes, pitch, flips, nflip, W, mask, nn, np, bits);
}

// Diagonal of M' K_S (sum over the subset's GRM markers of z'^2, the Jacobi preconditioner's
// Get_Diagof_StdGeno, FIT.cpp:665-704), lut4[4 m + code] = d'_m (g - 2p'_m)^2 per packed code (the
// missing code carries the subset fill).  Pass 1: block = 256 words of a marker row (16 samples
// each, so a warp reads 128 contiguous bytes) x a chunk of kDiagChunkM markers.  The table is
// staged 256 markers at a time in shared memory as pair entries: entry n of a marker holds the
// values of the two samples whose codes form the 4-bit field n, so one 8-byte shared load serves two
// samples.  FP32 sums per chunk into part[chunk][sample], each sample's markers added in marker
// order; the words of eight marker rows are requested together.  Pass 2: per sample, the chunks'
// partials added in chunk order in FP64.
constexpr int kDiagChunkM = 1024;
// 256 threads and a 32 KB table stage.  (128-thread blocks with a 16 KB stage fit on an SM beside a
// genotype-GEMM CTA, but measured 0.9% lower bench throughput than these in an A/B on one GPU.)
constexpr int kDiagThreads = 256;

__global__ void __launch_bounds__(kDiagThreads)
subset_diag_part_kernel(const uint32_t* __restrict__ codes32, int64_t words_per_row, int64_t nwords,
                        const float4* __restrict__ lut4, int64_t m, int64_t np, float* __restrict__ part) {
  __shared__ float2 spair[kDiagThreads][16];
  const int64_t w = (int64_t)blockIdx.x * kDiagThreads + threadIdx.x;
  const int64_t m0 = (int64_t)blockIdx.y * kDiagChunkM;
  const int64_t m1 = m0 + kDiagChunkM < m ? m0 + kDiagChunkM : m;
  float acc[16];
#pragma unroll
  for (int s = 0; s < 16; ++s) acc[s] = 0.0f;
  for (int64_t k0 = m0; k0 < m1; k0 += kDiagThreads) {
    const int kn = (int)(m1 - k0 < kDiagThreads ? m1 - k0 : kDiagThreads);
    __syncthreads();
    // entry i = (marker i / 16, field i % 16): a warp writes 32 consecutive entries (no bank conflicts)
    for (int i = threadIdx.x; i < 16 * kn; i += kDiagThreads) {
      const float4 q = __ldg(lut4 + k0 + (i >> 4));
      const int n = i & 15;
      const float a = (n & 3) == 0 ? q.x : (n & 3) == 1 ? q.y : (n & 3) == 2 ? q.z : q.w;
      const float b = (n >> 2) == 0 ? q.x : (n >> 2) == 1 ? q.y : (n >> 2) == 2 ? q.z : q.w;
      spair[i >> 4][n] = make_float2(a, b);
    }
    __syncthreads();
    if (w < nwords) {
      const uint32_t* row = codes32 + k0 * words_per_row + w;
      // eight marker rows' words requested together, then added in marker order
      int k = 0;
      for (; k + 8 <= kn; k += 8) {
        uint32_t word[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) word[u] = __ldg(row + (int64_t)(k + u) * words_per_row);
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const float2* e = spair[k + u];
#pragma unroll
          for (int s = 0; s < 16; s += 2) {
            const float2 v = e[(word[u] >> (2 * s)) & 15u];
            acc[s] += v.x;
            acc[s + 1] += v.y;
          }
        }
      }
      for (; k < kn; ++k) {
        const uint32_t word = __ldg(row + (int64_t)k * words_per_row);
        const float2* e = spair[k];
#pragma unroll
        for (int s = 0; s < 16; s += 2) {
          const float2 v = e[(word >> (2 * s)) & 15u];
          acc[s] += v.x;
          acc[s + 1] += v.y;
        }
      }
    }
  }
  if (w < nwords) {
    float* out = part + (int64_t)blockIdx.y * np + 16 * w;
#pragma unroll
    for (int s = 0; s < 16; ++s)
      if (16 * w + s < np) out[s] = acc[s];
  }
}

__global__ void subset_diag_sum_kernel(const float* __restrict__ part, int nchunks, int64_t nn, int64_t np,
                                       double* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  double t = 0.0;
  if (i < nn)
    for (int c = 0; c < nchunks; ++c) t += (double)part[(int64_t)c * np + i];
  out[i] = t;
}

int64_t subset_diag_scratch(int64_t m, int64_t np) { return ((m + kDiagChunkM - 1) / kDiagChunkM) * np; }

void launch_subset_diag(const uint8_t* codes, int64_t pitch, const float* lut4, int64_t m, int64_t nn, int64_t np,
                        float* part, double* out, cudaStream_t s) {
  const int64_t nwords = (nn + 15) / 16;
  const int nchunks = (int)((m + kDiagChunkM - 1) / kDiagChunkM);
  if (nchunks > 0 && nwords > 0) {
    dim3 grid((unsigned)((nwords + kDiagThreads - 1) / kDiagThreads), (unsigned)nchunks);
    subset_diag_part_kernel<<<grid, kDiagThreads, 0, s>>>(reinterpret_cast<const uint32_t*>(codes), pitch / 4, nwords,
                                                      reinterpret_cast<const float4*>(lut4), m, np, part);
  }
  subset_diag_sum_kernel<<<(unsigned)((np + kThreads - 1) / kThreads), kThreads, 0, s>>>(part, nchunks, nn, np, out);
}

// ----------------------------------------------------------------------------------- per step
// FP64 arithmetic is a small fraction of this GPU's FP32 rate, so the per-element work below runs
// in FP32: each thread sums its kChunk / kThreads elements in FP32 and the block adds the threads'
// partials in FP64, in a fixed order.
//
// Column sums over the subset (rows outside S are zero in P): block partials, kChunk rows each.
// With pmax, also the block's max |P| (the FP16 form scales each column by a power of two).
__global__ void subset_colsum_kernel(const float* __restrict__ Pf, int64_t np, const int32_t* __restrict__ cols,
                                     double* __restrict__ part, float* __restrict__ pmax, int nblk) {
  __shared__ double sh[kThreads / 32];
  __shared__ float shm[kThreads / 32];
  const int64_t j = blockIdx.y;
  const int32_t col = cols[j];
  const int64_t i0 = (int64_t)blockIdx.x * kChunk;
  float v = 0.0f, mx = 0.0f;
  if (col >= 0) {
    const float* p = Pf + (int64_t)col * np;
    for (int64_t i = i0 + threadIdx.x; i < i0 + kChunk && i < np; i += kThreads) {
      v += p[i];
      mx = fmaxf(mx, fabsf(p[i]));
    }
  }
  const double vd = block_sum((double)v, sh);
  if (threadIdx.x == 0) part[j * nblk + blockIdx.x] = vd;
  if (pmax) {
    const float bm = block_max(mx, shm);
    if (threadIdx.x == 0) pmax[j * nblk + blockIdx.x] = bm;
  }
}

// v_c = P - mean_S(P) on the subset (0 elsewhere and for padding columns), as BF16 high + low
// halves of the compact block (column j at row j * np).
__global__ void subset_center_split_kernel(const float* __restrict__ Pf, int64_t np, const int32_t* __restrict__ cols,
                                           const ColState* __restrict__ st, const SubsetSlot* __restrict__ slots,
                                           const double* __restrict__ winv, const double* __restrict__ part,
                                           int nblk, __nv_bfloat16* __restrict__ Vh, __nv_bfloat16* __restrict__ Vl) {
  __shared__ float s_mu;
  const int64_t j = blockIdx.y;
  const int32_t col = cols[j];
  const int64_t i0 = (int64_t)blockIdx.x * kChunk;
  int slot = 0;
  if (col >= 0) slot = st[col].pheno;
  if (threadIdx.x == 0) {
    double sum = 0.0;
    if (col >= 0)
      for (int b = 0; b < nblk; ++b) sum += part[j * nblk + b];
    s_mu = col >= 0 ? (float)(sum / slots[slot].ns) : 0.0f;
  }
  __syncthreads();
  const float mu = s_mu;
  for (int64_t i = i0 + threadIdx.x; i < i0 + kChunk && i < np; i += kThreads) {
    float v = 0.0f;
    if (col >= 0 && winv[(int64_t)slot * np + i] != 0.0) v = Pf[(int64_t)col * np + i] - mu;
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    Vh[j * np + i] = h;
    Vl[j * np + i] = __float2bfloat16_rn(v - __bfloat162float(h));
  }
}

// T[j, flips[k]] += dfill[k] * sum over the subset samples missing at that marker of v_c[j, i]:
// block (j, w) scans every sample's bit-map word w and accumulates the (at most 32) markers of that
// word in registers, then reduces them over the block in a fixed order.
__global__ void subset_flip_t_kernel(const __nv_bfloat16* __restrict__ Vh, const __nv_bfloat16* __restrict__ Vl,
                                     int64_t np, int64_t nn, const int32_t* __restrict__ cols,
                                     const ColState* __restrict__ st, const SubsetSlot* __restrict__ slots,
                                     float* __restrict__ T, int64_t mg) {
  __shared__ float red[kThreads / 32][32];
  const int64_t j = blockIdx.y;
  const int32_t col = cols[j];
  if (col < 0) return;
  const SubsetSlot sl = slots[st[col].pheno];
  const int w = blockIdx.x;
  if (w >= sl.W) return;
  float acc[32];
#pragma unroll
  for (int b = 0; b < 32; ++b) acc[b] = 0.0f;
  const uint32_t* bw = sl.bits + (int64_t)w * np;
  for (int64_t i = threadIdx.x; i < nn; i += kThreads) {
    const uint32_t word = bw[i];
    if (word == 0u) continue;
    const float v = __bfloat162float(Vh[j * np + i]) + __bfloat162float(Vl[j * np + i]);
#pragma unroll
    for (int b = 0; b < 32; ++b)
      if ((word >> b) & 1u) acc[b] += v;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int b = 0; b < 32; ++b) {
    float x = acc[b];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == b) red[warp][b] = x;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const int b = threadIdx.x;
    const int k = 32 * w + b;
    if (k < sl.nflip) {
      float s = 0.0f;
      for (int q = 0; q < kThreads / 32; ++q) s += red[q][b];
      T[j * mg + sl.flips[k]] += sl.dfill[k] * s;
    }
  }
}

// T' = d' .* T as BF16 high + low halves (compact block, column j at row j * mg), and the block
// partials of (2p')^T T' in FP64 (from the halves GEMM 2 multiplies).  Padding columns get zeros.
__global__ void subset_scale_split_kernel(const float* __restrict__ T, int64_t mg, const int32_t* __restrict__ cols,
                                          const ColState* __restrict__ st, const SubsetSlot* __restrict__ slots,
                                          __nv_bfloat16* __restrict__ Th, __nv_bfloat16* __restrict__ Tl,
                                          double* __restrict__ part, int nblk) {
  __shared__ double sh[kThreads / 32];
  const int64_t j = blockIdx.y;
  const int32_t col = cols[j];
  const int64_t m0 = (int64_t)blockIdx.x * kChunk;
  const SubsetSlot* sl = col >= 0 ? &slots[st[col].pheno] : nullptr;
  float cf = 0.0f;
  for (int64_t mk = m0 + threadIdx.x; mk < m0 + kChunk && mk < mg; mk += kThreads) {
    float t = 0.0f;
    if (sl) t = sl->dprime[mk] * T[j * mg + mk];
    const __nv_bfloat16 h = __float2bfloat16_rn(t);
    const __nv_bfloat16 l = __float2bfloat16_rn(t - __bfloat162float(h));
    Th[j * mg + mk] = h;
    Tl[j * mg + mk] = l;
    // h + l is exact in FP32 (16 significant bits): the value GEMM 2 multiplies
    if (sl) cf = fmaf(sl->p2[mk], __bfloat162float(h) + __bfloat162float(l), cf);
  }
  const double c = block_sum((double)cf, sh);
  if (threadIdx.x == 0) part[j * nblk + blockIdx.x] = c;
}

// K_S v on the subset: (U + dF T' - (2p')^T T') / M', written to column cols[j] of Y (zero outside
// the subset); padding columns are skipped.  The fill-flip term of sample i sums, over the flip
// markers k at which i is missing (set bits of the slot's word-major bit map), dfill[k] T'[j, flips[k]];
// those products are staged per column in shared memory, kFinF flips (kFinF / 32 bit-map words) at a
// time, so the scattered reads of T' happen once per block, not once per missing genotype.  The
// terms (a few tens per sample) are added in ascending flip order.
constexpr int kFinF = 2048;
constexpr int kFinPer = kChunk / kThreads;  // samples per thread

__global__ void __launch_bounds__(kThreads)
subset_finalize_kernel(const float* __restrict__ U, int64_t np, int64_t nn, const int32_t* __restrict__ cols,
                       const ColState* __restrict__ st, const SubsetSlot* __restrict__ slots,
                       const __nv_bfloat16* __restrict__ Th, const __nv_bfloat16* __restrict__ Tl, int64_t mg,
                       const double* __restrict__ part, int nblk, const double* __restrict__ winv,
                       float* __restrict__ Yf) {
  __shared__ double s_c;
  __shared__ float tf[kFinF];
  const int64_t j = blockIdx.y;
  const int32_t col = cols[j];
  if (col < 0) return;
  const int slot = st[col].pheno;
  const SubsetSlot sl = slots[slot];
  if (threadIdx.x == 0) {
    double c = 0.0;
    for (int b = 0; b < nblk; ++b) c += part[j * nblk + b];
    s_c = c;
  }
  const int64_t i0 = (int64_t)blockIdx.x * kChunk + threadIdx.x;
  unsigned live = 0u;
#pragma unroll
  for (int r = 0; r < kFinPer; ++r) {
    const int64_t i = i0 + (int64_t)r * kThreads;
    if (i < nn && winv[(int64_t)slot * np + i] != 0.0) live |= 1u << r;
  }
  float du[kFinPer];
#pragma unroll
  for (int r = 0; r < kFinPer; ++r) du[r] = 0.0f;
  const __nv_bfloat16* th = Th + j * mg;
  const __nv_bfloat16* tl = Tl + j * mg;
  for (int f0 = 0; f0 < sl.nflip; f0 += kFinF) {
    const int fn = sl.nflip - f0 < kFinF ? sl.nflip - f0 : kFinF;
    __syncthreads();
    for (int k = threadIdx.x; k < fn; k += kThreads) {
      const int64_t mk = sl.flips[f0 + k];
      tf[k] = sl.dfill[f0 + k] * (__bfloat162float(th[mk]) + __bfloat162float(tl[mk]));
    }
    __syncthreads();
    const int w0 = f0 / 32, wn = (fn + 31) / 32;
#pragma unroll
    for (int r = 0; r < kFinPer; ++r) {
      if (!((live >> r) & 1u)) continue;
      const uint32_t* bw = sl.bits + (int64_t)w0 * np + i0 + (int64_t)r * kThreads;
      float d = du[r];
      for (int w = 0; w < wn; ++w) {
        uint32_t word = bw[(int64_t)w * np];
        while (word) {
          const int b = __ffs(word) - 1;
          word &= word - 1u;
          d += tf[32 * w + b];
        }
      }
      du[r] = d;
    }
  }
  __syncthreads();
  const float cf = (float)s_c, inv_mf = (float)sl.inv_m;
#pragma unroll
  for (int r = 0; r < kFinPer; ++r) {
    const int64_t i = i0 + (int64_t)r * kThreads;
    if (i >= np) break;
    float y = 0.0f;
    if ((live >> r) & 1u) y = (U[j * np + i] - cf + du[r]) * inv_mf;
    Yf[(int64_t)col * np + i] = y;
  }
}

int subset_nblk(int64_t n) { return (int)((n + kChunk - 1) / kChunk); }

// ------------------------------------------------------- FP16-high / E4M3-low form of the same step
// The same data flow with per-column power-of-two scales: v_c s1 is split into FP16 + E4M3 halves;
// GEMM 1 gives T s1; T' s2 = d' T s1 (s2 / s1) is split the same way; GEMM 2 gives U s2, and the
// finalize divides s2 out.  scale[j] = s1, scale[cap + j] = s2 of compact column j.

__global__ void subset_center_split_f8_kernel(const float* __restrict__ Pf, int64_t np, const int32_t* __restrict__ cols,
                                              const ColState* __restrict__ st, const SubsetSlot* __restrict__ slots,
                                              const double* __restrict__ winv, const double* __restrict__ part,
                                              const float* __restrict__ pmax, int nblk, __half* __restrict__ Vh,
                                              uint8_t* __restrict__ Vl, float* __restrict__ scale) {
  __shared__ float s_mu, s_sc;
  const int64_t j = blockIdx.y;
  const int32_t col = cols[j];
  const int64_t i0 = (int64_t)blockIdx.x * kChunk;
  int slot = 0;
  if (col >= 0) slot = st[col].pheno;
  if (threadIdx.x == 0) {
    double sum = 0.0;
    float mx = 0.0f;
    if (col >= 0)
      for (int b = 0; b < nblk; ++b) {
        sum += part[j * nblk + b];
        mx = fmaxf(mx, pmax[j * nblk + b]);
      }
    const float mu = col >= 0 ? (float)(sum / slots[slot].ns) : 0.0f;
    s_mu = mu;
    s_sc = pow2_scale(mx + fabsf(mu));  // bounds |P - mu| over the column
    if (blockIdx.x == 0) scale[j] = s_sc;
  }
  __syncthreads();
  const float mu = s_mu, sc = s_sc;
  for (int64_t i = i0 + threadIdx.x; i < i0 + kChunk && i < np; i += kThreads) {
    float v = 0.0f;
    if (col >= 0 && winv[(int64_t)slot * np + i] != 0.0) v = (Pf[(int64_t)col * np + i] - mu) * sc;
    __half h;
    uint8_t l;
    split_f8(v, h, l);
    Vh[j * np + i] = h;
    Vl[j * np + i] = l;
  }
}

// Fill-change corrections of T s1 (as subset_flip_t_kernel, over the scaled halves).
__global__ void subset_flip_t_f8_kernel(const __half* __restrict__ Vh, const uint8_t* __restrict__ Vl, int64_t np,
                                        int64_t nn, const int32_t* __restrict__ cols, const ColState* __restrict__ st,
                                        const SubsetSlot* __restrict__ slots, float* __restrict__ T, int64_t mg) {
  __shared__ float red[kThreads / 32][32];
  const int64_t j = blockIdx.y;
  const int32_t col = cols[j];
  if (col < 0) return;
  const SubsetSlot sl = slots[st[col].pheno];
  const int w = blockIdx.x;
  if (w >= sl.W) return;
  float acc[32];
#pragma unroll
  for (int b = 0; b < 32; ++b) acc[b] = 0.0f;
  const uint32_t* bw = sl.bits + (int64_t)w * np;
  for (int64_t i = threadIdx.x; i < nn; i += kThreads) {
    const uint32_t word = bw[i];
    if (word == 0u) continue;
    const float v = join_f8(Vh[j * np + i], Vl[j * np + i]);
#pragma unroll
    for (int b = 0; b < 32; ++b)
      if ((word >> b) & 1u) acc[b] += v;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int b = 0; b < 32; ++b) {
    float x = acc[b];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == b) red[warp][b] = x;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const int b = threadIdx.x;
    const int k = 32 * w + b;
    if (k < sl.nflip) {
      float s = 0.0f;
      for (int q = 0; q < kThreads / 32; ++q) s += red[q][b];
      T[j * mg + sl.flips[k]] += sl.dfill[k] * s;
    }
  }
}

// Block maxima of |d' T s1| (for s2).
__global__ void subset_tmax_kernel(const float* __restrict__ T, int64_t mg, const int32_t* __restrict__ cols,
                                   const ColState* __restrict__ st, const SubsetSlot* __restrict__ slots,
                                   float* __restrict__ pmax, int nblk) {
  __shared__ float shm[kThreads / 32];
  const int64_t j = blockIdx.y;
  const int32_t col = cols[j];
  const int64_t m0 = (int64_t)blockIdx.x * kChunk;
  float mx = 0.0f;
  if (col >= 0) {
    const SubsetSlot* sl = &slots[st[col].pheno];
    for (int64_t mk = m0 + threadIdx.x; mk < m0 + kChunk && mk < mg; mk += kThreads)
      mx = fmaxf(mx, fabsf(sl->dprime[mk] * T[j * mg + mk]));
  }
  const float bm = block_max(mx, shm);
  if (threadIdx.x == 0) pmax[j * nblk + blockIdx.x] = bm;
}

// T' s2 = d' (T s1) (s2 / s1) as FP16 + E4M3 halves, and the block partials of (2p')^T T'.
__global__ void subset_scale_split_f8_kernel(const float* __restrict__ T, int64_t mg, const int32_t* __restrict__ cols,
                                             const ColState* __restrict__ st, const SubsetSlot* __restrict__ slots,
                                             const float* __restrict__ pmax, float* __restrict__ scale, int64_t cap,
                                             __half* __restrict__ Th, uint8_t* __restrict__ Tl,
                                             double* __restrict__ part, int nblk) {
  __shared__ double sh[kThreads / 32];
  __shared__ float s_ratio, s_inv2;
  const int64_t j = blockIdx.y;
  const int32_t col = cols[j];
  const int64_t m0 = (int64_t)blockIdx.x * kChunk;
  const SubsetSlot* sl = col >= 0 ? &slots[st[col].pheno] : nullptr;
  if (threadIdx.x == 0) {
    float mx = 0.0f;
    for (int b = 0; b < nblk; ++b) mx = fmaxf(mx, pmax[j * nblk + b]);
    const float s1 = scale[j];
    const float s2 = pow2_scale(mx / s1);
    s_ratio = s2 / s1;
    s_inv2 = 1.0f / s2;
    if (blockIdx.x == 0) scale[cap + j] = s2;
  }
  __syncthreads();
  const float ratio = s_ratio;
  float cf = 0.0f;
  for (int64_t mk = m0 + threadIdx.x; mk < m0 + kChunk && mk < mg; mk += kThreads) {
    float t = 0.0f;
    if (sl) t = sl->dprime[mk] * T[j * mg + mk] * ratio;
    __half h;
    uint8_t l;
    split_f8(t, h, l);
    Th[j * mg + mk] = h;
    Tl[j * mg + mk] = l;
    if (sl) cf = fmaf(sl->p2[mk], join_f8(h, l), cf);
  }
  const double c = block_sum((double)cf, sh);
  if (threadIdx.x == 0) part[j * nblk + blockIdx.x] = c * (double)s_inv2;
}

__global__ void __launch_bounds__(kThreads)
subset_finalize_f8_kernel(const float* __restrict__ U, int64_t np, int64_t nn, const int32_t* __restrict__ cols,
                          const ColState* __restrict__ st, const SubsetSlot* __restrict__ slots,
                          const __half* __restrict__ Th, const uint8_t* __restrict__ Tl, int64_t mg,
                          const float* __restrict__ scale2, const double* __restrict__ part, int nblk,
                          const double* __restrict__ winv, float* __restrict__ Yf) {
  __shared__ double s_c;
  __shared__ float tf[kFinF];
  const int64_t j = blockIdx.y;
  const int32_t col = cols[j];
  if (col < 0) return;
  const int slot = st[col].pheno;
  const SubsetSlot sl = slots[slot];
  if (threadIdx.x == 0) {
    double c = 0.0;
    for (int b = 0; b < nblk; ++b) c += part[j * nblk + b];
    s_c = c;
  }
  const float inv2 = 1.0f / scale2[j];
  const int64_t i0 = (int64_t)blockIdx.x * kChunk + threadIdx.x;
  unsigned live = 0u;
#pragma unroll
  for (int r = 0; r < kFinPer; ++r) {
    const int64_t i = i0 + (int64_t)r * kThreads;
    if (i < nn && winv[(int64_t)slot * np + i] != 0.0) live |= 1u << r;
  }
  float du[kFinPer];
#pragma unroll
  for (int r = 0; r < kFinPer; ++r) du[r] = 0.0f;
  const __half* th = Th + j * mg;
  const uint8_t* tl = Tl + j * mg;
  for (int f0 = 0; f0 < sl.nflip; f0 += kFinF) {
    const int fn = sl.nflip - f0 < kFinF ? sl.nflip - f0 : kFinF;
    __syncthreads();
    for (int k = threadIdx.x; k < fn; k += kThreads) {
      const int64_t mk = sl.flips[f0 + k];
      tf[k] = sl.dfill[f0 + k] * (join_f8(th[mk], tl[mk]) * inv2);
    }
    __syncthreads();
    const int w0 = f0 / 32, wn = (fn + 31) / 32;
#pragma unroll
    for (int r = 0; r < kFinPer; ++r) {
      if (!((live >> r) & 1u)) continue;
      const uint32_t* bw = sl.bits + (int64_t)w0 * np + i0 + (int64_t)r * kThreads;
      float d = du[r];
      for (int w = 0; w < wn; ++w) {
        uint32_t word = bw[(int64_t)w * np];
        while (word) {
          const int b = __ffs(word) - 1;
          word &= word - 1u;
          d += tf[32 * w + b];
        }
      }
      du[r] = d;
    }
  }
  __syncthreads();
  const float cf = (float)s_c, inv_mf = (float)sl.inv_m;
#pragma unroll
  for (int r = 0; r < kFinPer; ++r) {
    const int64_t i = i0 + (int64_t)r * kThreads;
    if (i >= np) break;
    float y = 0.0f;
    if ((live >> r) & 1u) y = (U[j * np + i] * inv2 - cf + du[r]) * inv_mf;
    Yf[(int64_t)col * np + i] = y;
  }
}

void launch_subset_prepare_f8(const float* Pf, int64_t np, const int32_t* cols, int64_t ncols, const ColState* st,
                              const SubsetSlot* slots, const double* winv, double* part, float* pmax, void* Vh,
                              void* Vl, float* scale, cudaStream_t s) {
  const int nblk = subset_nblk(np);
  dim3 grid((unsigned)nblk, (unsigned)ncols);
  subset_colsum_kernel<<<grid, kThreads, 0, s>>>(Pf, np, cols, part, pmax, nblk);
  subset_center_split_f8_kernel<<<grid, kThreads, 0, s>>>(Pf, np, cols, st, slots, winv, part, pmax, nblk,
                                                          static_cast<__half*>(Vh), static_cast<uint8_t*>(Vl),
                                                          scale);
}

void launch_subset_scale_f8(const void* Vh, const void* Vl, int64_t np, int64_t nn, const int32_t* cols,
                            int64_t ncols, const ColState* st, const SubsetSlot* slots, int max_w, float* T,
                            int64_t mg, void* Th, void* Tl, double* part, float* pmax, float* scale, int64_t cap,
                            cudaStream_t s) {
  if (max_w > 0) {
    dim3 g1((unsigned)max_w, (unsigned)ncols);
    subset_flip_t_f8_kernel<<<g1, kThreads, 0, s>>>(static_cast<const __half*>(Vh), static_cast<const uint8_t*>(Vl),
                                                    np, nn, cols, st, slots, T, mg);
  }
  const int nblk = subset_nblk(mg);
  dim3 g2((unsigned)nblk, (unsigned)ncols);
  subset_tmax_kernel<<<g2, kThreads, 0, s>>>(T, mg, cols, st, slots, pmax, nblk);
  subset_scale_split_f8_kernel<<<g2, kThreads, 0, s>>>(T, mg, cols, st, slots, pmax, scale, cap,
                                                       static_cast<__half*>(Th), static_cast<uint8_t*>(Tl), part,
                                                       nblk);
}

void launch_subset_finalize_f8(const float* U, int64_t np, int64_t nn, const int32_t* cols, int64_t ncols,
                               const ColState* st, const SubsetSlot* slots, const void* Th, const void* Tl,
                               int64_t mg, const float* scale2, const double* part, const double* winv, float* Yf,
                               cudaStream_t s) {
  dim3 grid((unsigned)subset_nblk(np), (unsigned)ncols);
  subset_finalize_f8_kernel<<<grid, kThreads, 0, s>>>(U, np, nn, cols, st, slots, static_cast<const __half*>(Th),
                                                      static_cast<const uint8_t*>(Tl), mg, scale2, part,
                                                      subset_nblk(mg), winv, Yf);
}



void launch_subset_prepare(const float* Pf, int64_t np, const int32_t* cols, int64_t ncols, const ColState* st,
                           const SubsetSlot* slots, const double* winv, double* part, void* Vh, void* Vl,
                           cudaStream_t s) {
  const int nblk = subset_nblk(np);
  dim3 grid((unsigned)nblk, (unsigned)ncols);
  subset_colsum_kernel<<<grid, kThreads, 0, s>>>(Pf, np, cols, part, nullptr, nblk);
  subset_center_split_kernel<<<grid, kThreads, 0, s>>>(Pf, np, cols, st, slots, winv, part, nblk,
                                                       static_cast<__nv_bfloat16*>(Vh),
                                                       static_cast<__nv_bfloat16*>(Vl));
}

void launch_subset_scale(const void* Vh, const void* Vl, int64_t np, int64_t nn, const int32_t* cols, int64_t ncols,
                         const ColState* st, const SubsetSlot* slots, int max_w, float* T, int64_t mg, void* Th,
                         void* Tl, double* part, cudaStream_t s) {
  if (max_w > 0) {
    dim3 g1((unsigned)max_w, (unsigned)ncols);
    subset_flip_t_kernel<<<g1, kThreads, 0, s>>>(static_cast<const __nv_bfloat16*>(Vh),
                                                 static_cast<const __nv_bfloat16*>(Vl), np, nn, cols, st, slots, T,
                                                 mg);
  }
  const int nblk = subset_nblk(mg);
  dim3 g2((unsigned)nblk, (unsigned)ncols);
  subset_scale_split_kernel<<<g2, kThreads, 0, s>>>(T, mg, cols, st, slots, static_cast<__nv_bfloat16*>(Th),
                                                    static_cast<__nv_bfloat16*>(Tl), part, nblk);
}

void launch_subset_finalize(const float* U, int64_t np, int64_t nn, const int32_t* cols, int64_t ncols,
                            const ColState* st, const SubsetSlot* slots, const void* Th, const void* Tl, int64_t mg,
                            const double* part, const double* winv, float* Yf, cudaStream_t s) {
  dim3 grid((unsigned)subset_nblk(np), (unsigned)ncols);
  subset_finalize_kernel<<<grid, kThreads, 0, s>>>(U, np, nn, cols, st, slots, static_cast<const __nv_bfloat16*>(Th),
                                                   static_cast<const __nv_bfloat16*>(Tl), mg, part, subset_nblk(mg),
                                                   winv, Yf);
}

}  // namespace sg
