// Genotype kernels: PLINK .bed decode + per-marker QC, re-pack, standardisation,
// GRM diagonal, and the synthetic-cohort generator.
//
// The integer work (allele / missing counts, re-pack) is bit-exact with the
// reference genoClass (src/SAIGE/src/SAIGE_fitGLMM_fast.cpp, FIT.cpp below);
// the float work (frequencies, 1/sd, LUT, FP32 diagonal) uses explicitly
// rounded IEEE intrinsics so it is bit-exact with the reference's float code.
// These are HBM-bound byte kernels: 16-byte aligned row pitches, 32-bit word
// loads and popcounts; no tensor cores.
#include "sg_internal.h"
#include <cuda_bf16.h>
#include <math.h>

namespace sg {

// ----------------------------------------------------------------------------
// Per-marker counts and QC: one warp per marker.
// 2-bit field f of sample s: b = bit0, a = bit1; 00 -> 2, 01 -> missing,
// 10 -> 1, 11 -> 0 (FIT.cpp:346-357).  With lo = b bits and hi = a bits of a
// 32-bit word (16 samples): missing = lo & ~hi; a non-missing sample adds
// 2 - (a + b) alleles.  ``maskbits`` has bit 2s set for samples with a
// phenotype (indicatorGenoSamplesWithPheno, FIT.cpp:376-385).
// ----------------------------------------------------------------------------
__global__ void marker_qc_kernel(const uint8_t* __restrict__ raw, int64_t pitch, int64_t m,
                                 int64_t n_fam, const uint32_t* __restrict__ maskbits, int64_t nn,
                                 float min_maf, float max_miss, const uint8_t* __restrict__ vr_flag,
                                 float min_mac_vr, float max_mac_vr, int is_var_ratio,
                                 MarkerQC* __restrict__ out) {
  const int64_t marker = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (marker >= m) return;
  const uint32_t* row = reinterpret_cast<const uint32_t*>(raw + marker * pitch);
  const int64_t nwords = (n_fam + 15) / 16;
  int nnon = 0, nmiss = 0, sum_ab = 0;
  auto count = [&](uint32_t x, uint32_t mk) {
    const uint32_t lo = x & 0x55555555u, hi = (x >> 1) & 0x55555555u;
    const uint32_t miss = lo & ~hi;
    const uint32_t non = ~miss & mk;
    nmiss += __popc(miss & mk);
    nnon += __popc(non);
    sum_ab += __popc(hi & non) + __popc(lo & non);
  };
  // 16-byte loads over the row's whole quads (rows start 16-byte aligned), then the last words;
  // the mask's quads need the same alignment, which cudaMalloc gives
  const int64_t nquads = nwords / 4;
  const uint4* row4 = reinterpret_cast<const uint4*>(row);
  const uint4* mk4 = reinterpret_cast<const uint4*>(maskbits);
  for (int64_t q = lane; q < nquads; q += 32) {
    const uint4 x = __ldg(row4 + q), mk = __ldg(mk4 + q);
    count(x.x, mk.x);
    count(x.y, mk.y);
    count(x.z, mk.z);
    count(x.w, mk.w);
  }
  for (int64_t w = 4 * nquads + lane; w < nwords; w += 32) count(__ldg(row + w), __ldg(maskbits + w));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    nnon += __shfl_xor_sync(0xffffffffu, nnon, o);
    nmiss += __shfl_xor_sync(0xffffffffu, nmiss, o);
    sum_ab += __shfl_xor_sync(0xffffffffu, sum_ab, o);
  }
  if (lane != 0) return;
  int allele = 2 * nnon - sum_ab;
  // FIT.cpp:436-447: first frequency over non-missing calls, integer fill
  const float alt0 = __fdiv_rn((float)allele, (float)((nn - nmiss) * 2));
  const float miss_rate = __fdiv_rn((float)nmiss, (float)nn);
  int fill = 0;
  if (isfinite(alt0)) fill = (int)floor((double)__fmul_rn(2.0f, alt0) + 0.5);
  if (nmiss > 0) allele = allele + fill * nmiss;  // FIT.cpp:449-454
  const float alt = __fdiv_rn((float)allele, (float)(nn * 2));  // FIT.cpp:484
  const float maf = fminf(alt, __fsub_rn(1.0f, alt));
  const int mac = min(allele, (int)(nn * 2) - allele);
  int pass_qc = (maf >= min_maf && miss_rate <= max_miss) ? 1 : 0;  // FIT.cpp:493-495
  int pass_vr = 0;
  if (is_var_ratio) {
    if (max_mac_vr != -1.0f) {
      // categorical variance ratios (FIT.cpp:497-518): every marker with min <= MAC < max, and the
      // random draw's markers from max up
      if ((float)mac >= min_mac_vr && (float)mac < max_mac_vr) pass_vr = 1;
      else if ((float)mac >= max_mac_vr && vr_flag[marker]) pass_vr = 1;
    } else if ((float)mac >= min_mac_vr && vr_flag[marker]) {
      pass_vr = 1;  // FIT.cpp:521-543
    }
  }
  if (pass_vr) pass_qc = 0;                                                      // FIT.cpp:545-547
  // FIT.cpp:916-921: Std = sqrt(2p(1-p)), invStd = 1/Std (0 if Std == 0), in float
  const float sd = __fsqrt_rn(__fmul_rn(__fmul_rn(2.0f, alt), __fsub_rn(1.0f, alt)));
  const float inv = (sd == 0.0f) ? 0.0f : __fdiv_rn(1.0f, sd);
  MarkerQC q;
  q.allele = allele;
  q.mac = mac;
  q.nmiss = nmiss;
  q.freq = alt;
  q.invstd = inv;
  q.fill = fill;
  q.pass_qc = pass_qc;
  q.pass_vr = pass_vr;
  out[marker] = q;
}

void launch_marker_qc(const uint8_t* raw, int64_t raw_pitch, int64_t m, int64_t n_fam,
                      const uint32_t* maskbits, int64_t nn, float min_maf, float max_miss,
                      const uint8_t* vr_flag, float min_mac_vr, float max_mac_vr, int is_var_ratio,
                      MarkerQC* out, cudaStream_t s) {
  const int warps = 8;
  const int64_t blocks = (m + warps - 1) / warps;
  if (blocks == 0) return;
  marker_qc_kernel<<<(unsigned)blocks, warps * 32, 0, s>>>(raw, raw_pitch, m, n_fam, maskbits, nn,
                                                          min_maf, max_miss, vr_flag, min_mac_vr,
                                                          max_mac_vr, is_var_ratio, out);
}

// ----------------------------------------------------------------------------
// Re-pack (FIT.cpp:551-575): for output marker j (source marker src_marker[j]),
// sample k takes the source field of sample sub0[k]; a missing field (01)
// becomes the code of the fill genotype.  The reference's re-pack codes
// (HOM_ALT=11, HET=10, HOM_REF=00) equal the source fields for non-missing
// calls, so only missing fields change.  Fields past nn and the row padding
// are zero.
// ----------------------------------------------------------------------------
__device__ __forceinline__ uint32_t pack_code_of(int g) { return g == 0 ? 3u : (g == 1 ? 2u : 0u); }

__global__ void repack_gather_kernel(const uint8_t* __restrict__ raw, int64_t raw_pitch,
                                     const int32_t* __restrict__ src_marker,
                                     const MarkerQC* __restrict__ qc, const int32_t* __restrict__ sub0,
                                     int64_t nn, uint8_t* __restrict__ out, int64_t out_pitch) {
  const int64_t j = blockIdx.y;
  const int64_t byte = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (byte >= out_pitch) return;
  const int64_t src = src_marker[j];
  const uint8_t* row = raw + src * raw_pitch;
  const uint32_t fcode = qc ? pack_code_of(qc[src].fill) : 1u;  // no qc: missing calls stay 01
  uint32_t v = 0;
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const int64_t k = byte * 4 + t;
    if (k < nn) {
      const int64_t si = sub0[k];
      uint32_t f = (row[si >> 2] >> (2 * (si & 3))) & 3u;
      if (f == 1u) f = fcode;
      v |= f << (2 * t);
    }
  }
  out[j * out_pitch + byte] = (uint8_t)v;
}

// Identity sample order (nn == n_fam, sub0[k] == k): 32-bit word at a time.
__global__ void repack_identity_kernel(const uint8_t* __restrict__ raw, int64_t raw_pitch,
                                       const int32_t* __restrict__ src_marker,
                                       const MarkerQC* __restrict__ qc, int64_t nn,
                                       uint8_t* __restrict__ out, int64_t out_pitch) {
  const int64_t j = blockIdx.y;
  const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nwords = out_pitch / 4;
  if (w >= nwords) return;
  const int64_t src = src_marker[j];
  const uint32_t* row = reinterpret_cast<const uint32_t*>(raw + src * raw_pitch);
  const uint32_t fcode = qc ? pack_code_of(qc[src].fill) : 1u;  // no qc: missing calls stay 01
  uint32_t x = row[w];
  // valid-sample mask of this word (bits of both halves of each field)
  const int64_t s0 = w * 16;
  uint32_t valid;
  if (s0 + 16 <= nn) valid = 0xffffffffu;
  else if (s0 >= nn) valid = 0u;
  else valid = (1u << (2 * (nn - s0))) - 1u;
  const uint32_t lo = x & 0x55555555u, hi = (x >> 1) & 0x55555555u;
  const uint32_t miss = lo & ~hi;
  x = (x & ~(miss * 3u)) | (miss * fcode);
  reinterpret_cast<uint32_t*>(out + j * out_pitch)[w] = x & valid;
}

void launch_repack(const uint8_t* raw, int64_t raw_pitch, const int32_t* src_marker,
                   const MarkerQC* qc, int64_t m_out, const int32_t* sub0, int64_t nn, int identity,
                   uint8_t* out, int64_t out_pitch, cudaStream_t s) {
  if (m_out == 0) return;
  const int threads = 256;
  for (int64_t j0 = 0; j0 < m_out; j0 += 65535) {
    const int64_t mj = (m_out - j0) < 65535 ? (m_out - j0) : 65535;
    if (identity) {
      dim3 grid((unsigned)((out_pitch / 4 + threads - 1) / threads), (unsigned)mj);
      repack_identity_kernel<<<grid, threads, 0, s>>>(raw, raw_pitch, src_marker + j0, qc, nn,
                                                      out + j0 * out_pitch, out_pitch);
    } else {
      dim3 grid((unsigned)((out_pitch + threads - 1) / threads), (unsigned)mj);
      repack_gather_kernel<<<grid, threads, 0, s>>>(raw, raw_pitch, src_marker + j0, qc, sub0, nn,
                                                    out + j0 * out_pitch, out_pitch);
    }
  }
}

// LUT (g - 2p) * invStd for g = 0,1,2 (setStdGenoLookUpArr FIT.cpp:152-159), in float.
__global__ void lut_kernel(const MarkerQC* __restrict__ qc, const int32_t* __restrict__ src_marker,
                           int64_t m_out, float* __restrict__ lut4) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m_out) return;
  const MarkerQC q = qc[src_marker[j]];
  const float p2 = __fmul_rn(2.0f, q.freq);
  lut4[4 * j + 0] = __fmul_rn(__fsub_rn(0.0f, p2), q.invstd);
  lut4[4 * j + 1] = __fmul_rn(__fsub_rn(1.0f, p2), q.invstd);
  lut4[4 * j + 2] = __fmul_rn(__fsub_rn(2.0f, p2), q.invstd);
  lut4[4 * j + 3] = 0.0f;
}

void launch_lut(const MarkerQC* qc, const int32_t* src_marker, int64_t m_out, float* lut4,
                cudaStream_t s) {
  if (m_out == 0) return;
  lut_kernel<<<(unsigned)((m_out + 255) / 256), 256, 0, s>>>(qc, src_marker, m_out, lut4);
}

// genotype 0/1/2 of a re-packed field (Get_OneSNP_StdGeno FIT.cpp:620-628: 2 - (a + b))
__device__ __forceinline__ int field_geno(uint32_t f) { return 2 - (int)((f & 1u) + (f >> 1)); }

// ----------------------------------------------------------------------------
// Standardised genotypes Z (np x mp): row = sample, markers contiguous, zero
// padded.  Block = 64 markers x 128 samples staged through shared memory so
// the transposing writes are coalesced along markers.
// ----------------------------------------------------------------------------
template <typename Out>
__global__ void zbuild_kernel(const uint8_t* __restrict__ packed, int64_t pitch,
                              const float* __restrict__ lut4, int64_t m_qc, int64_t nn,
                              int64_t mp, Out* __restrict__ Zhi, Out* __restrict__ Zlo) {
  __shared__ uint32_t sbytes[64][9];  // 64 markers x 32 bytes (+pad)
  __shared__ float slut[64][4];
  const int64_t m0 = (int64_t)blockIdx.x * 64;
  const int64_t s0 = (int64_t)blockIdx.y * 128;
  const int tid = threadIdx.x;
  for (int e = tid; e < 64 * 8; e += blockDim.x) {
    const int mm = e >> 3, wd = e & 7;
    const int64_t mk = m0 + mm;
    const int64_t boff = s0 / 4 + (int64_t)wd * 4;
    uint32_t v = 0;
    if (mk < m_qc && boff < pitch) v = *reinterpret_cast<const uint32_t*>(packed + mk * pitch + boff);
    sbytes[mm][wd] = v;
  }
  for (int e = tid; e < 64 * 4; e += blockDim.x) {
    const int mm = e >> 2;
    const int64_t mk = m0 + mm;
    slut[mm][e & 3] = (mk < m_qc) ? lut4[mk * 4 + (e & 3)] : 0.0f;
  }
  __syncthreads();
  const int mm = tid & 63;
  const int64_t mk = m0 + mm;
  for (int s = tid >> 6; s < 128; s += (blockDim.x >> 6)) {
    const int64_t smp = s0 + s;
    float z = 0.0f;
    if (mk < m_qc && smp < nn) {
      const uint32_t f = (sbytes[mm][s >> 4] >> (2 * (s & 15))) & 3u;
      z = slut[mm][field_geno(f)];
    }
    if constexpr (sizeof(Out) == 4) {
      Zhi[smp * mp + mk] = z;
    } else {
      const __nv_bfloat16 h = __float2bfloat16_rn(z);
      Zhi[smp * mp + mk] = h;
      if (Zlo) Zlo[smp * mp + mk] = __float2bfloat16_rn(z - __bfloat162float(h));
    }
  }
}

void launch_zbuild_f32(const uint8_t* packed, int64_t pitch, const float* lut4, int64_t m_qc,
                       int64_t nn, int64_t np, int64_t mp, float* Z, cudaStream_t s) {
  dim3 grid((unsigned)(mp / 64), (unsigned)(np / 128));
  zbuild_kernel<float><<<grid, 256, 0, s>>>(packed, pitch, lut4, m_qc, nn, mp, Z, nullptr);
}
void launch_zbuild_bf16(const uint8_t* packed, int64_t pitch, const float* lut4, int64_t m_qc,
                        int64_t nn, int64_t np, int64_t mp, void* Zhi, void* Zlo, cudaStream_t s) {
  dim3 grid((unsigned)(mp / 64), (unsigned)(np / 128));
  zbuild_kernel<__nv_bfloat16><<<grid, 256, 0, s>>>(packed, pitch, lut4, m_qc, nn, mp,
                                                   (__nv_bfloat16*)Zhi, (__nv_bfloat16*)Zlo);
}

// Marker-major standardised genotypes Zm (m_rows x np, samples contiguous), zero past nn and for
// padding rows >= m (LOCO correction operand).
__global__ void zbuild_marker_major_kernel(const uint8_t* __restrict__ packed, int64_t pitch,
                                           const float* __restrict__ lut4, int64_t m, int64_t nn,
                                           int64_t np, float* __restrict__ Zm) {
  const int64_t row = blockIdx.y;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  float z = 0.0f;
  if (row < m && i < nn) {
    const uint32_t f = (packed[row * pitch + (i >> 2)] >> (2 * (i & 3))) & 3u;
    z = lut4[4 * row + field_geno(f)];
  }
  Zm[row * np + i] = z;
}

void launch_zbuild_marker_major(const uint8_t* packed, int64_t pitch, const float* lut4, int64_t m,
                                int64_t m_rows, int64_t nn, int64_t np, float* Zm, cudaStream_t s) {
  if (m_rows == 0) return;
  dim3 grid((unsigned)((np + 255) / 256), (unsigned)m_rows);
  zbuild_marker_major_kernel<<<grid, 256, 0, s>>>(packed, pitch, lut4, m, nn, np, Zm);
}

// Y = (a * Y - V) * b elementwise over ncols x np (LOCO: (M K P - Z_j Z_j' P) / (M - M_j))
__global__ void loco_combine_f32_kernel(float* Y, const float* __restrict__ V, float a, float b, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) Y[i] = (a * Y[i] - V[i]) * b;
}
__global__ void loco_combine_f64_kernel(double* Y, const float* __restrict__ V, double a, double b, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) Y[i] = (a * Y[i] - (double)V[i]) * b;
}
void launch_loco_combine(float* Yf, double* Yd, const float* V, double a, double b, int64_t n,
                         cudaStream_t s) {
  if (n == 0) return;
  if (Yf) loco_combine_f32_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(Yf, V, (float)a, (float)b, n);
  else loco_combine_f64_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(Yd, V, a, b, n);
}

// ----------------------------------------------------------------------------
// GRM diagonal sum_m z^2 (Get_Diagof_StdGeno FIT.cpp:665-704).
//
// FP32: markers in order per sample, rounded exactly as the reference's
// ``m_DiagStd + z % z`` (z*z rounded to FP32, then added), so each sample's
// chain is sequential in m.  Beside it the high-precision diagonal is
// accumulated in unsigned 64-bit fixed point: lutq[4m + g] = round(z^2 2^F)
// with F chosen by the host so that no sum can overflow; integer sums are
// exact and order-independent, and F ~ 39 at M = 150k keeps each term to
// 2^-40.  Both per-marker tables (z*z in FP32 and the fixed-point square) are
// built once, so the per-sample loop is two table reads and two adds.
//
// Layout: one thread per sample; a block owns 128 consecutive bytes of every
// marker row (512 samples) and streams the rows and the two tables through
// shared memory in chunks of 128 markers with cp.async double buffering.
// ----------------------------------------------------------------------------
__global__ void diag_tables_kernel(const float* __restrict__ lut4, int64_t m, double scale,
                                   unsigned long long* __restrict__ lutq, float* __restrict__ lutsq) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= 4 * m) return;
  const float z = lut4[j];
  lutsq[j] = __fmul_rn(z, z);
  const double zd = (double)z;
  lutq[j] = __double2ull_rn(zd * zd * scale);  // zd*zd is exact in FP64, the scale a power of two
}

constexpr int kDiagBytes = 128;                // byte columns per block
constexpr int kDiagThreads = 4 * kDiagBytes;   // one sample per thread
constexpr int kDiagChunk = 128;                // markers per staged chunk

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, int src_bytes) {
  const uint32_t d = static_cast<uint32_t>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(gmem), "r"(src_bytes) : "memory");
}

__global__ void __launch_bounds__(kDiagThreads)
diag_kernel(const uint8_t* __restrict__ packed, int64_t pitch, const unsigned long long* __restrict__ lutq,
            const float* __restrict__ lutsq, int64_t m_qc, int64_t nn, double inv_scale,
            double* __restrict__ d64, float* __restrict__ d32) {
  __shared__ __align__(16) uint8_t tile[2][kDiagChunk][kDiagBytes];        // 32 KB
  __shared__ __align__(16) float ssq[2][kDiagChunk][4];                    // 4 KB
  __shared__ __align__(16) unsigned long long sq[2][kDiagChunk][4];        // 8 KB
  const int t = threadIdx.x;
  const int64_t col0 = (int64_t)blockIdx.x * kDiagBytes;
  // per chunk: 1024 row pieces + 128 FP32-table pieces + 256 fixed-point-table pieces (16 B each);
  // pieces past the row's pitch or the last marker are zero-filled without a global read
  auto issue = [&](int buf, int64_t m0) {
    for (int idx = t; idx < 1024 + 128 + 256; idx += kDiagThreads) {
      if (idx < 1024) {
        const int r = idx >> 3, q = idx & 7;
        const int64_t mk = m0 + r;
        const int64_t col = col0 + q * 16;
        const bool ok = mk < m_qc && col + 16 <= pitch;
        cp_async16(&tile[buf][r][q * 16], ok ? packed + mk * pitch + col : packed, ok ? 16 : 0);
      } else if (idx < 1024 + 128) {
        const int r = idx - 1024;
        const bool ok = m0 + r < m_qc;
        cp_async16(&ssq[buf][r][0], ok ? lutsq + 4 * (m0 + r) : lutsq, ok ? 16 : 0);
      } else {
        const int e = idx - 1024 - 128, r = e >> 1, h = e & 1;
        const bool ok = m0 + r < m_qc;
        cp_async16(&sq[buf][r][2 * h], ok ? lutq + 4 * (m0 + r) + 2 * h : lutq, ok ? 16 : 0);
      }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  const int byte = t >> 2, sh = 2 * (t & 3);
  float a32 = 0.0f;
  unsigned long long aq = 0ull;
  const int64_t nchunks = (m_qc + kDiagChunk - 1) / kDiagChunk;
  if (nchunks > 0) issue(0, 0);
  for (int64_t c = 0; c < nchunks; ++c) {
    if (c + 1 < nchunks) {
      issue((int)((c + 1) & 1), (c + 1) * kDiagChunk);
      asm volatile("cp.async.wait_group 1;" ::: "memory");
    } else {
      asm volatile("cp.async.wait_group 0;" ::: "memory");
    }
    __syncthreads();
    const int buf = (int)(c & 1);
    const int64_t m0 = c * kDiagChunk;
    const int rows = (int)(m_qc - m0 < kDiagChunk ? m_qc - m0 : kDiagChunk);
#pragma unroll 4
    for (int r = 0; r < rows; ++r) {
      const int g = field_geno((tile[buf][r][byte] >> sh) & 3u);
      a32 = __fadd_rn(a32, ssq[buf][r][g]);
      aq += sq[buf][r][g];
    }
    __syncthreads();  // the buffer is refilled by the next chunk's copies
  }
  const int64_t i = col0 * 4 + t;
  if (i < nn) {
    d32[i] = a32;
    d64[i] = (double)aq * inv_scale;
  }
}

void launch_diag(const uint8_t* packed, int64_t pitch, const float* lut4, int64_t m_qc, int64_t nn,
                 int frac_bits, void* scratch, double* diag64, float* diag32, cudaStream_t s) {
  if (nn == 0) return;
  const double scale = ldexp(1.0, frac_bits);
  unsigned long long* lutq = static_cast<unsigned long long*>(scratch);
  float* lutsq = reinterpret_cast<float*>(lutq + 4 * m_qc);
  if (m_qc > 0)
    diag_tables_kernel<<<(unsigned)((4 * m_qc + 255) / 256), 256, 0, s>>>(lut4, m_qc, scale, lutq, lutsq);
  const int64_t nbytes = (nn + 3) / 4;
  diag_kernel<<<(unsigned)((nbytes + kDiagBytes - 1) / kDiagBytes), kDiagThreads, 0, s>>>(
      packed, pitch, lutq, lutsq, m_qc, nn, 1.0 / scale, diag64, diag32);
}

// One marker unpacked to genotypes and standardised values (Get_OneSNP_Geno / _StdGeno).
__global__ void unpack_marker_kernel(const uint8_t* __restrict__ row, int64_t nn,
                                     const float* __restrict__ lut4, int32_t* g, float* z) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn) return;
  const uint32_t f = (row[i >> 2] >> (2 * (i & 3))) & 3u;
  const int gg = field_geno(f);
  if (g) g[i] = gg;
  if (z) z[i] = lut4 ? lut4[gg] : 0.0f;
}

void launch_unpack_marker(const uint8_t* packed_row, int64_t nn, const float* lut4, int32_t* g,
                          float* z, cudaStream_t s) {
  if (nn == 0) return;
  unpack_marker_kernel<<<(unsigned)((nn + 255) / 256), 256, 0, s>>>(packed_row, nn, lut4, g, z);
}

// ----------------------------------------------------------------------------
// Synthetic cohort (integer recipe, reproduced on the CPU by saigegpu/synth.py):
//   hm  = hash3(seed, 1, m);  thr_m = 167772 + (((hm >> 40) * 8220835) >> 24)   (p_m in [0.01,0.5))
//   h   = hash3(seed, 16 + m, i); allele1 = (h >> 40) < thr_m; allele2 = ((h >> 16) & 0xFFFFFF) < thr_m
//   missing when (h & 0xFFFF) < miss_thr16; genotype g = allele1 + allele2 copies of the counted allele
//   field: missing 01, g=2 -> 00, g=1 -> 10, g=0 -> 11.
// ----------------------------------------------------------------------------
__device__ __forceinline__ uint32_t synth_field(uint64_t seed, int64_t m, int64_t i, uint32_t thr,
                                                uint32_t miss_thr16) {
  const uint64_t h = hash3(seed, 16ull + (uint64_t)m, (uint64_t)i);
  if ((uint32_t)(h & 0xFFFFu) < miss_thr16) return 1u;
  const int g = (int)((uint32_t)(h >> 40) < thr) + (int)((uint32_t)((h >> 16) & 0xFFFFFFu) < thr);
  return g == 2 ? 0u : (g == 1 ? 2u : 3u);
}

__global__ void synth_bed_kernel(uint64_t seed, int64_t n, int64_t m, uint32_t miss_thr16,
                                 uint8_t* __restrict__ body, int64_t nb) {
  const int64_t marker = blockIdx.y + (int64_t)blockIdx.z * 65535;
  const int64_t byte = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (marker >= m || byte >= nb) return;
  const uint64_t hm = hash3(seed, 1ull, (uint64_t)marker);
  const uint32_t thr = 167772u + (uint32_t)(((hm >> 40) * 8220835ull) >> 24);
  uint32_t v = 0;
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const int64_t i = byte * 4 + t;
    if (i < n) v |= synth_field(seed, marker, i, thr, miss_thr16) << (2 * t);
  }
  body[marker * nb + byte] = (uint8_t)v;
}

void launch_synth_bed(uint64_t seed, int64_t n, int64_t m, uint32_t miss_thr16, uint8_t* out,
                      cudaStream_t s) {
  const int64_t nb = (n + 3) / 4;
  const int threads = 256;
  const int64_t gz = (m + 65534) / 65535;
  dim3 grid((unsigned)((nb + threads - 1) / threads), (unsigned)(m < 65535 ? m : 65535), (unsigned)gz);
  synth_bed_kernel<<<grid, threads, 0, s>>>(seed, n, m, miss_thr16, out + 3, nb);
}

// Per-marker effect b_m ~ N(0,1) (Box-Muller on two 53-bit hash uniforms).
__global__ void effect_kernel(uint64_t seed, int64_t m, float* b) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m) return;
  const double u1 = ((double)(hash3(seed, 2ull, (uint64_t)j) >> 11) + 0.5) * 0x1.0p-53;
  const double u2 = (double)(hash3(seed, 3ull, (uint64_t)j) >> 11) * 0x1.0p-53;
  b[j] = (float)(sqrt(-2.0 * log(u1)) * cospi(2.0 * u2));
}

__global__ void genetic_value_kernel(const uint8_t* __restrict__ packed, int64_t pitch,
                                     const float* __restrict__ lut4, int64_t m_qc, int64_t nn,
                                     const float* __restrict__ b, double* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn) return;
  const int64_t byte = i >> 2;
  const int sh = 2 * (int)(i & 3);
  double acc = 0.0;
  for (int64_t m = 0; m < m_qc; ++m) {
    const uint32_t f = (packed[m * pitch + byte] >> sh) & 3u;
    acc += (double)__ldg(lut4 + 4 * m + field_geno(f)) * (double)__ldg(b + m);
  }
  out[i] = acc / sqrt((double)m_qc);
}

void launch_genetic_value(const uint8_t* packed, int64_t pitch, const float* lut4, int64_t m_qc,
                          int64_t nn, uint64_t seed, double* out, cudaStream_t s) {
  float* b = nullptr;
  if (cudaMallocAsync(&b, sizeof(float) * (m_qc > 0 ? m_qc : 1), s) != cudaSuccess) return;
  effect_kernel<<<(unsigned)((m_qc + 255) / 256), 256, 0, s>>>(seed, m_qc, b);
  genetic_value_kernel<<<(unsigned)((nn + 127) / 128), 128, 0, s>>>(packed, pitch, lut4, m_qc, nn,
                                                                    b, out);
  cudaFreeAsync(b, s);
}

}  // namespace sg
