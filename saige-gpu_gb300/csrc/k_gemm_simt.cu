// CUDA-core GEMMs of the GRM path.
//
// gemm_nt: C = scale * A B^T with A (M x K) and B (N x K) both row-major with
// the reduction dimension contiguous -- the layout of the standardised
// genotypes Z (sample rows, markers contiguous), of the GRM K (symmetric) and
// of a block of RHS-major vectors.  One kernel therefore serves the exact
// FP32 SYRK (K = Z Z^T / M over lower-triangle tiles, mirrored) and the FP32
// multi-RHS GRM.V (Y^T = K P^T).  Block tile 128 x BN x 8, 256 threads, an
// 8 x (BN/16) register tile per thread, double-buffered shared memory.
//
// gemv_f64: y = K x with FP64 products and sums, one warp per row -- the plain
// FP64 single-RHS matvec used by the baseline PCG path.
#include "sg_internal.h"
#include <math.h>

namespace sg {

template <int BN>
__global__ void __launch_bounds__(256)
gemm_nt_kernel(const float* __restrict__ A, int64_t lda, const float* __restrict__ B, int64_t ldb,
               float* __restrict__ C, int64_t ldc, int64_t K, float scale, int mode) {
  constexpr int BM = 128, BK = 8, TM = 8, TN = BN / 16;
  __shared__ __align__(16) float As[2][BK][BM + 4];
  __shared__ __align__(16) float Bs[2][BK][BN + 4];
  int64_t bi, bj;
  if (mode == 2) {
    // lower-triangle tile index t -> (bi, bj), bj <= bi
    const int64_t t = blockIdx.x;
    int64_t r = (int64_t)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while ((r + 1) * (r + 2) / 2 <= t) ++r;
    while (r * (r + 1) / 2 > t) --r;
    bi = r;
    bj = t - r * (r + 1) / 2;
  } else {
    bi = blockIdx.y;
    bj = blockIdx.x;
  }
  const float* Ab = A + bi * BM * lda;
  const float* Bb = B + bj * BN * ldb;
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int a_row = tid >> 1, a_k = (tid & 1) * 4;
  const bool b_loader = tid < BN * 2;
  const int b_row = tid >> 1, b_k = (tid & 1) * 4;

  float acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = 0.0f;

  float4 ra = *reinterpret_cast<const float4*>(Ab + (int64_t)a_row * lda + a_k);
  float4 rb = make_float4(0.f, 0.f, 0.f, 0.f);
  if (b_loader) rb = *reinterpret_cast<const float4*>(Bb + (int64_t)b_row * ldb + b_k);
  int buf = 0;
  As[0][a_k + 0][a_row] = ra.x; As[0][a_k + 1][a_row] = ra.y;
  As[0][a_k + 2][a_row] = ra.z; As[0][a_k + 3][a_row] = ra.w;
  if (b_loader) {
    Bs[0][b_k + 0][b_row] = rb.x; Bs[0][b_k + 1][b_row] = rb.y;
    Bs[0][b_k + 2][b_row] = rb.z; Bs[0][b_k + 3][b_row] = rb.w;
  }
  __syncthreads();
  for (int64_t k0 = 0; k0 < K; k0 += BK) {
    const bool more = (k0 + BK) < K;
    if (more) {
      ra = *reinterpret_cast<const float4*>(Ab + (int64_t)a_row * lda + k0 + BK + a_k);
      if (b_loader) rb = *reinterpret_cast<const float4*>(Bb + (int64_t)b_row * ldb + k0 + BK + b_k);
    }
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      float a[TM], b[TN];
      const float4 a0 = *reinterpret_cast<const float4*>(&As[buf][kk][ty * TM]);
      const float4 a1 = *reinterpret_cast<const float4*>(&As[buf][kk][ty * TM + 4]);
      a[0] = a0.x; a[1] = a0.y; a[2] = a0.z; a[3] = a0.w;
      a[4] = a1.x; a[5] = a1.y; a[6] = a1.z; a[7] = a1.w;
#pragma unroll
      for (int j = 0; j < TN; j += 2) {
        const float2 bb = *reinterpret_cast<const float2*>(&Bs[buf][kk][tx * TN + j]);
        b[j] = bb.x; b[j + 1] = bb.y;
      }
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    if (more) {
      const int nb = buf ^ 1;
      As[nb][a_k + 0][a_row] = ra.x; As[nb][a_k + 1][a_row] = ra.y;
      As[nb][a_k + 2][a_row] = ra.z; As[nb][a_k + 3][a_row] = ra.w;
      if (b_loader) {
        Bs[nb][b_k + 0][b_row] = rb.x; Bs[nb][b_k + 1][b_row] = rb.y;
        Bs[nb][b_k + 2][b_row] = rb.z; Bs[nb][b_k + 3][b_row] = rb.w;
      }
      __syncthreads();
      buf = nb;
    }
  }
  const int64_t r0 = bi * BM + ty * TM;
  const int64_t c0 = bj * BN + tx * TN;
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const float v = acc[i][j] * scale;
      const int64_t r = r0 + i, c = c0 + j;
      if (mode == 1) {
        C[c * ldc + r] = v;
      } else {
        C[r * ldc + c] = v;
        if (mode == 2 && bi != bj) C[c * ldc + r] = v;
      }
    }
}

void launch_gemm_nt_f32(const float* A, int64_t lda, const float* B, int64_t ldb, float* C,
                        int64_t ldc, int64_t M, int64_t N, int64_t K, float scale, int mode,
                        cudaStream_t s) {
  if (M == 0 || N == 0) return;
  if (mode == 2) {
    const int64_t nt = M / 128;
    gemm_nt_kernel<128><<<(unsigned)(nt * (nt + 1) / 2), 256, 0, s>>>(A, lda, B, ldb, C, ldc, K,
                                                                      scale, 2);
    return;
  }
  if (N % 128 == 0 && N >= 256) {
    dim3 grid((unsigned)(N / 128), (unsigned)(M / 128));
    gemm_nt_kernel<128><<<grid, 256, 0, s>>>(A, lda, B, ldb, C, ldc, K, scale, mode);
  } else if (N % 64 == 0) {
    dim3 grid((unsigned)(N / 64), (unsigned)(M / 128));
    gemm_nt_kernel<64><<<grid, 256, 0, s>>>(A, lda, B, ldb, C, ldc, K, scale, mode);
  } else {
    dim3 grid((unsigned)(N / 32), (unsigned)(M / 128));
    gemm_nt_kernel<32><<<grid, 256, 0, s>>>(A, lda, B, ldb, C, ldc, K, scale, mode);
  }
}

__global__ void gemv_f64_kernel(const float* __restrict__ K, int64_t ld, int64_t n,
                                const double* __restrict__ x, double* __restrict__ y) {
  const int64_t row = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  const float4* kr = reinterpret_cast<const float4*>(K + row * ld);
  const double2* x2 = reinterpret_cast<const double2*>(x);
  double acc = 0.0;
  for (int64_t j = lane; j < n / 4; j += 32) {
    const float4 k = __ldg(kr + j);
    const double2 xa = x2[2 * j], xb = x2[2 * j + 1];
    acc = fma((double)k.x, xa.x, acc);
    acc = fma((double)k.y, xa.y, acc);
    acc = fma((double)k.z, xb.x, acc);
    acc = fma((double)k.w, xb.y, acc);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) y[row] = acc;
}

void launch_gemv_f64(const float* K, int64_t ld, int64_t n, const double* x, double* y,
                     cudaStream_t s) {
  if (n == 0) return;
  gemv_f64_kernel<<<(unsigned)((n + 7) / 8), 256, 0, s>>>(K, ld, n, x, y);
}

}  // namespace sg
