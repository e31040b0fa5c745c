// tcgen05 (5th-generation tensor core) GEMMs of the GRM path, sm_103a.
//
//   D[128 x BN] (+)= A[128 x K] * B[BN x K]^T,  A and B K-major in global memory
//
// One CTA computes one 128 x BN output tile over the whole reduction:
//   warp 8 (one lane)  TMA producer: cp.async.bulk.tensor 2D loads of 128-byte
//                      wide K slices (SWIZZLE_128B) into an S-stage ring,
//                      completion tracked by mbarrier transaction counts;
//   warp 9 (one lane)  MMA issuer: tcgen05.mma.cta_group::1 with shared-memory
//                      descriptors into one of two FP32 accumulators in TMEM
//                      (128 lanes x BN columns each); tcgen05.commit frees each
//                      stage and hands over each finished accumulator;
//                      warp 9 also allocates / frees the TMEM columns;
//   warps 0-7          drain: tcgen05.ld 32x32b of each finished accumulator
//                      (warp w: TMEM lanes 32 (w % 4).. = 32 output rows, every
//                      other 32-column group), added into FP32 registers, then
//                      scale and store to global after the last one.
// Drained accumulation: accumulating into TMEM loses magnitude -- measured, a
// sum over the whole reduction (tens of thousands of MMAs at N = 100k) came out
// 1e-4 to 3e-4 smaller than the FP64 value, a bias that grows linearly with the
// reduction length, as rounding each accumulation toward zero would give.
// Here an accumulator covers only 512 bytes of K per row (16 MMA K steps per
// product) before it is added, round-to-nearest, into registers, while the
// MMAs fill the other accumulator.  Measured at N = 100k against an
// FP64 GEMV on the same K, the split-BF16 GRM.V's bias went from -1e-4..-3e-4
// to -3e-7..-8e-7 relative, and a binary fit's tau from 1.1% off to 3e-5; the
// launches are 3% (1024 columns) to 13% (384 columns) slower, the SYRK 8%.
// (256-byte chunks: bias below 4.3e-7, launches 8-19% slower.)
// Optional CTA pairs (2-CTA clusters, tcgen05 cta_group::2) compute 256-row tiles: each CTA loads
// its own operand rows with plain TMA loads, so a pair reads half the B bytes per SM (see the
// kernel's kPair parameter).  The drain length is a launch argument (option SG_TC_DRAIN_BYTES,
// 512 bytes by default).  Every mbarrier wait is bounded by a global-timer budget; on expiry the
// kernel records an error code, skips the remaining work, waits for the MMAs it issued, frees its
// TMEM and returns.
//
// Uses:
//   * SYRK  K = scale * Z Z^T (Z bf16, kind::f16): lower-triangle tiles only,
//     each element (r, c <= r) written to K[r][c] and K[c][r].  The split
//     variant accumulates all four products of Z = Zh + Zl.
//   * GRM.V Y^T = K P^T (K fp32 read as tf32, kind::tf32), output stored
//     RHS-major so each TMEM column is a coalesced row of Y^T; split variants
//     with TF32 or BF16 high/low halves of K and P (three products).
#include "sg_internal.h"
#include <algorithm>

#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

namespace sg {

namespace {

constexpr int kTileM = 128;
// products per K step of the GEMM kernel (see tc_gemm_kernel)
constexpr int kOne = 0, kSplitB = 1, kSplit3 = 2, kSplit4 = 3, kSplitB8 = 4;
// operands of the second products (A2, B2) exist for every form but kOne (B2) and kSplitB (A2)
__host__ __device__ constexpr bool form_has_a2(int f) { return f == kSplit3 || f == kSplit4 || f == kSplitB8; }
__host__ __device__ constexpr bool form_has_b2(int f) { return f != kOne; }
// row bytes of the second operands per stage: kSplitB8's are E4M3, half the bytes of FP16 A and B
__host__ __device__ constexpr int form_rb2(int f, int rb) { return f == kSplitB8 ? rb / 2 : rb; }
constexpr int kRowBytes = 128;                 // one SWIZZLE_128B atom row
constexpr int kATileBytes = kTileM * kRowBytes;  // 16 KB
constexpr unsigned long long kWaitBudgetNs = 4000000000ull;  // 4 s per wait
// warp roles of the GEMM kernel: 8 drain/epilogue warps, the TMA producer, the MMA issuer
constexpr int kDrainWarps = 8;
constexpr int kProducerWarp = 8;
constexpr int kMmaWarp = 9;
constexpr int kGemmThreads = 320;

__device__ int g_tc_error = 0;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.b32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: returns false (and records ``code``) when the budget runs out
// or another thread of this kernel already gave up.
__device__ __forceinline__ bool mbar_wait_budget(uint64_t* bar, uint32_t parity, int code,
                                                 volatile int* abort_flag, unsigned long long budget_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = gtimer();
  for (uint32_t it = 1;; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 255u) == 0u) {
      if (*abort_flag) return false;
      if (gtimer() - t0 > budget_ns) {
        *abort_flag = 1;
        atomicCAS(&g_tc_error, 0, code);
        return false;
      }
    }
  }
}

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int code,
                                          volatile int* abort_flag) {
  return mbar_wait_budget(bar, parity, code, abort_flag, kWaitBudgetNs);
}

// Bounded wait with a sleeping back-off between polls, for waits that last a whole chunk of MMAs:
// the drain warps share the SM's schedulers with the single-lane TMA and MMA loops.
__device__ __forceinline__ bool mbar_wait_sleep(uint64_t* bar, uint32_t parity, int code,
                                                volatile int* abort_flag) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = gtimer();
  unsigned ns = 32;
  for (;;) {
    __nanosleep(ns);
    if (mbar_try_wait(bar, parity)) return true;
    if (ns < 256) ns <<= 1;
    if (*abort_flag) return false;
    if (gtimer() - t0 > kWaitBudgetNs) {
      *abort_flag = 1;
      atomicCAS(&g_tc_error, 0, code);
      return false;
    }
  }
}

// Bounded wait at teardown: the MMAs a CTA issued complete within microseconds once issued (their
// operands are already in shared memory), so this wait ignores the abort flag and gives up after
// 1 s without recording anything.
__device__ __forceinline__ void mbar_wait_teardown(uint64_t* bar, uint32_t parity) {
  const unsigned long long t0 = gtimer();
  while (!mbar_try_wait(bar, parity))
    if (gtimer() - t0 > 1000000000ull) return;
}

// Self-test of the bounded wait: waits on an mbarrier that nothing arrives at, with a short budget,
// and reports through the same error flag the GEMM kernels use.
__global__ void wait_selftest_kernel(unsigned long long budget_ns, int* waited_out) {
  __shared__ __align__(8) uint64_t bar;
  __shared__ int abort_flag;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) *waited_out = mbar_wait_budget(&bar, 0u, 9, &abort_flag, budget_ns) ? 0 : 1;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar,
                                            int32_t x, int32_t y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];"
      ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y)
      : "memory");
}

// Shared-memory matrix descriptor, K-major operand in SWIZZLE_128B layout:
// start address >> 4 (bits 0-13), LBO unused for swizzled K-major (1),
// SBO = 1024 B between 8-row core-matrix groups (bits 32-45), descriptor
// version 1 (bits 46-47), layout SWIZZLE_128B = 2 (bits 61-63).
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// The same for K slices of RB bytes per row: SWIZZLE_128B (RB = 128) as above, or SWIZZLE_64B
// (RB = 64: SBO = 512 B between 8-row groups, layout code 4).
template <int RB>
__device__ __forceinline__ uint64_t smem_desc_kmajor(uint32_t addr) {
  if constexpr (RB == 128) {
    return smem_desc_sw128(addr);
  } else {
    uint64_t d = 0;
    d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)((8 * RB) >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)4 << 61;
    return d;
  }
}

// Instruction descriptor: FP32 accumulator, A/B format (1 = BF16 for
// kind::f16, 2 = TF32 for kind::tf32), both K-major, N >> 3 at bit 17,
// M >> 4 at bit 24 (M = 128 for one CTA, 256 for a CTA pair).
__host__ __device__ constexpr uint32_t make_idesc(uint32_t fmt, int m, int n) {
  return (1u << 4) | (fmt << 7) | (fmt << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(m >> 4) << 24);
}

template <bool kTF32, bool kPair>
__device__ __forceinline__ void umma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                     uint32_t accumulate) {
  if constexpr (kTF32 && kPair) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::2.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
  } else if constexpr (kTF32) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
  } else if constexpr (kPair) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
  } else {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
  }
}

// kind::f8f6f4 (both operands E4M3, K = 32 elements = 32 bytes per instruction, FP32 accumulator)
template <bool kPair>
__device__ __forceinline__ void umma_f8(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
  if constexpr (kPair) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::2.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
  } else {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
  }
}

__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Address of the same shared-memory location in CTA ``rank`` of the cluster.
__device__ __forceinline__ uint32_t cluster_addr(const void* p, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_u32(p)), "r"(rank));
  return r;
}

// Arrive once on an mbarrier given by its cluster address (this CTA's or the peer's).
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t bar_cluster) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(bar_cluster) : "memory");
}

// CTA-pair load: the box lands in this CTA's shared memory and completes its transaction bytes on
// the mbarrier at cluster address ``bar_cluster``, which may sit in the pair's other CTA.
__device__ __forceinline__ void tma_load_2d_pair(void* dst, const CUtensorMap* map, uint32_t bar_cluster,
                                                 int32_t x, int32_t y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4}], [%2];"
      ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(bar_cluster), "r"(x), "r"(y)
      : "memory");
}

template <bool kPair>
__device__ __forceinline__ void umma_commit(uint32_t bar_cluster) {
  if constexpr (kPair)
    asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 ::"r"(bar_cluster) : "memory");
  else
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 ::"r"(bar_cluster) : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
        "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
        "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

struct TileCoord {
  int32_t bm, bn;  // row block (128 rows; the first of two for a CTA pair) and column block (BN cols)
};

// kForm: the products accumulated per K step (operand halves come from the second maps):
//   kOne    A B                          (A and B loaded)
//   kSplitB A Bh + A Bl                  (A exact in the operand type, B as high + low halves)
//   kSplit3 Ah Bh + Ah Bl + Al Bh        (both as halves, the low x low term dropped)
//   kSplit4 Ah Bh + Ah Bl + Al Bh + Al Bl
//   kSplitB8 A Bh + A8 Bl8               (A, Bh in FP16 by kind::f16; A8 = A and Bl8 = the low half in
//                                         E4M3 by kind::f8f6f4, into the same accumulator; RB >= 256)
// kPair: two CTAs of a 2-CTA cluster compute one 256 x BN tile with tcgen05.mma.cta_group::2, issued
// by the even CTA (the leader).  Each CTA loads its own 128 rows of A and half of the B tile
// (BN / 2 rows) into the same shared-memory offsets with plain TMA loads; the loads of both signal
// the leader's full barrier (cta_group::2 form of the load), the leader's MMA commits arrive on the
// empty and accumulator barriers of each CTA (one commit addressed to each CTA), and each CTA drains
// its own 128 accumulator rows from its own TMEM.  Per SM this halves the B operand bytes read from
// L2 for the same tensor work.
// drain_kb: pipeline stages per TMEM accumulator chunk (the drain length is drain_kb * RB bytes of
// K per row).  Rows >= nrows of a tile (a padding row block) are not stored.
// RB: bytes of one operand row's K slice per pipeline stage -- 128 (SWIZZLE_128B) or 64
// (SWIZZLE_64B: half the bytes per stage, twice the stages in the same shared memory, for the
// split-BF16 GRM.V, whose four operand tiles per stage left it with only two stages of 128-byte
// slices), or 256 / 512: two / four adjacent 128-byte SWIZZLE_128B boxes per operand and stage, so
// that each stage reads 256 / 512 contiguous bytes of every operand row (more bytes per DRAM page
// opened when the rows of a streamed operand lie far apart, as G's do in the genotype GEMMs).
template <bool kTF32, int BN, int S, int kForm, bool kPair, int RB = 128>
__global__ void __launch_bounds__(kGemmThreads, 1)
tc_gemm_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
               const __grid_constant__ CUtensorMap mapA2, const __grid_constant__ CUtensorMap mapB2,
               const TileCoord* __restrict__ tiles, int num_kb, int drain_kb, float* __restrict__ D,
               int64_t ldd, float scale, int mode, int64_t nrows, const int32_t* __restrict__ colmap) {
  static_assert(RB == 512 || RB == 256 || RB == 128 || RB == 64, "K slices of 512, 256, 128 or 64 bytes");
  constexpr int kSW = RB > 128 ? 128 : RB;  // bytes of one swizzled box row (the TMA box's inner size)
  constexpr int kSub = RB / kSW;            // boxes per operand and stage, adjacent in K
  static_assert(!kPair || (BN / 2) % 8 == 0, "a CTA's half of the B tile is whole 8-row swizzle atoms");
  constexpr bool kF8 = kForm == kSplitB8;
  static_assert(!kF8 || (RB >= 256 && !kTF32), "the E4M3 low products take whole 128-byte boxes");
  constexpr int kATile = kTileM * RB;
  constexpr int kBRows = kPair ? BN / 2 : BN;  // rows of the B tile this CTA loads
  constexpr int kBTileBytes = kBRows * RB;
  constexpr int RB2 = form_rb2(kForm, RB);    // row bytes of A2 / B2 per stage
  constexpr int kSub2 = RB2 > 128 ? RB2 / 128 : 1;
  constexpr int kSW2 = RB2 > 128 ? 128 : RB2;
  constexpr int kATile2 = kTileM * RB2, kBTile2 = kBRows * RB2;
  constexpr int kStageBytes = kATile + kBTileBytes + (form_has_a2(kForm) ? kATile2 : 0) + (form_has_b2(kForm) ? kBTile2 : 0);
  // stage layout: [A][B][A2][B2], absent operands taking no room
  constexpr int kOffA2 = kATile + kBTileBytes;
  constexpr int kOffB2 = kOffA2 + (form_has_a2(kForm) ? kATile2 : 0);
  // operand formats: TF32 = 2, BF16 = 1, FP16 = 0 (kind::f16 / tf32); E4M3 = 0 (kind::f8f6f4)
  constexpr uint32_t kFmt = kTF32 ? 2u : (kF8 ? 0u : 1u);
  constexpr int kKSteps = RB / 32;     // 32 bytes of K per MMA
  constexpr int kKSteps2 = RB2 / 32;
  // two accumulators, each a power of two >= 32 columns wide
  constexpr uint32_t kAccCols = BN <= 32 ? 32 : BN <= 64 ? 64 : BN <= 128 ? 128 : 256;
  constexpr uint32_t kTmemCols = 2 * kAccCols;
  constexpr uint32_t kIdesc = make_idesc(kFmt, kPair ? 2 * kTileM : kTileM, BN);
  constexpr uint32_t kIdesc8 = make_idesc(0u, kPair ? 2 * kTileM : kTileM, BN);  // E4M3 x E4M3
  constexpr int kGroups = (BN + 31) / 32;     // 32-column groups of the tile
  constexpr int kHalfGroups = (kGroups + 1) / 2;
  static_assert(kDrainWarps == 8 && kGemmThreads == 32 * (kDrainWarps + 2),
                "two drain warps per TMEM lane quadrant, then the producer and MMA warps");
  static_assert(kTmemCols <= 512, "two accumulators of at most 256 columns");

  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + S * kStageBytes);
  uint64_t* empty = full + S;
  uint64_t* acc_full = empty + S;     // [2] the MMAs of an accumulator's chunk completed
  uint64_t* acc_empty = acc_full + 2;  // [2] the drain warps (of both CTAs of a pair) read the accumulator
  uint64_t* mma_done = acc_empty + 2;  // every MMA this CTA issued has completed (teardown)
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mma_done + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const uint32_t crank = kPair ? cluster_rank() : 0u;
  const bool leader = crank == 0;
  const TileCoord tc = tiles[kPair ? (blockIdx.x >> 1) : blockIdx.x];
  const int32_t row_block = tc.bm + (int32_t)crank;  // this CTA's 128 rows

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], kDrainWarps * (kPair ? 2 : 1));
    }
    mbar_init(mma_done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == kMmaWarp) {
    // a pair allocates collectively: one warp of each CTA, same columns, same address in both
    if constexpr (kPair) {
      asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;"
                   ::"r"(smem_u32(tmem_slot)), "r"(kTmemCols) : "memory");
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
    } else {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                   ::"r"(smem_u32(tmem_slot)), "r"(kTmemCols) : "memory");
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if constexpr (kPair) cluster_sync();  // both CTAs' barriers exist before either signals the other
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem_base = *tmem_slot;
  const int nchunks = (num_kb + drain_kb - 1) / drain_kb;

  if (warp == kProducerWarp) {
    if (lane == 0) {
      // ---------------- TMA producer (each CTA of a pair loads its own operand rows)
      const int32_t ya = row_block * kTileM, yb = tc.bn * BN + (int32_t)crank * kBRows;
      for (int kb = 0; kb < num_kb; ++kb) {
        const int s = kb % S;
        const uint32_t ph = (uint32_t)(kb / S) & 1u;
        if (!mbar_wait(&empty[s], ph ^ 1u, 1, abort_flag)) break;
        uint8_t* st = smem + s * kStageBytes;
        const int32_t x = kb * (RB / (kTF32 ? 4 : 2));
        // box u of an operand covers K bytes [u kSW, (u + 1) kSW) of the stage's slice and sits
        // u * rows * kSW bytes into the operand's region
        if constexpr (kPair) {
          // the leader's full barrier counts both CTAs' bytes; only the leader arrives on it
          const uint32_t fb = cluster_addr(&full[s], 0);
          if (leader) mbar_expect_tx(&full[s], 2u * (uint32_t)kStageBytes);
#pragma unroll
          for (int u = 0; u < kSub; ++u) {
            const int32_t xu = x + u * (kSW / (kTF32 ? 4 : 2));
            tma_load_2d_pair(st + u * kTileM * kSW, &mapA, fb, xu, ya);
            tma_load_2d_pair(st + kATile + u * kBRows * kSW, &mapB, fb, xu, yb);
            if constexpr (!kF8) {
              if constexpr (form_has_a2(kForm)) tma_load_2d_pair(st + kOffA2 + u * kTileM * kSW, &mapA2, fb, xu, ya);
              if constexpr (form_has_b2(kForm)) tma_load_2d_pair(st + kOffB2 + u * kBRows * kSW, &mapB2, fb, xu, yb);
            }
          }
          if constexpr (kF8) {  // E4M3 operands: one byte per element, the same K elements
#pragma unroll
            for (int u = 0; u < kSub2; ++u) {
              const int32_t xu = x + u * kSW2;
              tma_load_2d_pair(st + kOffA2 + u * kTileM * kSW2, &mapA2, fb, xu, ya);
              tma_load_2d_pair(st + kOffB2 + u * kBRows * kSW2, &mapB2, fb, xu, yb);
            }
          }
        } else {
          mbar_expect_tx(&full[s], (uint32_t)kStageBytes);
#pragma unroll
          for (int u = 0; u < kSub; ++u) {
            const int32_t xu = x + u * (kSW / (kTF32 ? 4 : 2));
            tma_load_2d(st + u * kTileM * kSW, &mapA, &full[s], xu, ya);
            tma_load_2d(st + kATile + u * kBRows * kSW, &mapB, &full[s], xu, yb);
            if constexpr (!kF8) {
              if constexpr (form_has_a2(kForm)) tma_load_2d(st + kOffA2 + u * kTileM * kSW, &mapA2, &full[s], xu, ya);
              if constexpr (form_has_b2(kForm)) tma_load_2d(st + kOffB2 + u * kBRows * kSW, &mapB2, &full[s], xu, yb);
            }
          }
          if constexpr (kF8) {
#pragma unroll
            for (int u = 0; u < kSub2; ++u) {
              const int32_t xu = x + u * kSW2;
              tma_load_2d(st + kOffA2 + u * kTileM * kSW2, &mapA2, &full[s], xu, ya);
              tma_load_2d(st + kOffB2 + u * kBRows * kSW2, &mapB2, &full[s], xu, yb);
            }
          }
        }
      }
    }
  } else if (warp == kMmaWarp) {
    if (lane == 0 && leader) {
      // ---------------- MMA issuer: chunk ch of drain_kb stages goes to accumulator ch % 2, which is
      // reused once the drain warps have read it (two chunks earlier)
      uint32_t empty_peer = 0, accf_peer = 0;
      if constexpr (kPair) {
        empty_peer = cluster_addr(empty, 1);
        accf_peer = cluster_addr(acc_full, 1);
      }
      for (int kb = 0; kb < num_kb; ++kb) {
        const int ch = kb / drain_kb;
        const int kin = kb - ch * drain_kb;
        const int ab = ch & 1;
        if (kin == 0) {
          if (!mbar_wait(&acc_empty[ab], ((uint32_t)(ch >> 1) & 1u) ^ 1u, 5, abort_flag)) break;
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        }
        const int s = kb % S;
        const uint32_t ph = (uint32_t)(kb / S) & 1u;
        if (!mbar_wait(&full[s], ph, 2, abort_flag)) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t dacc = tmem_base + (uint32_t)ab * kAccCols;
        const uint32_t a0 = smem_u32(smem + s * kStageBytes);
        const uint32_t b0 = a0 + kATile;
#pragma unroll
        for (int k = 0; k < kKSteps; ++k) {
          const uint32_t acc = (kin > 0 || k > 0) ? 1u : 0u;
          // 32 bytes of K per MMA: box k / (kSW / 32), offset 32 (k % (kSW / 32)) within its rows
          const uint32_t ka = (uint32_t)((k / (kSW / 32)) * kTileM * kSW + 32 * (k % (kSW / 32)));
          const uint32_t kbo = (uint32_t)((k / (kSW / 32)) * kBRows * kSW + 32 * (k % (kSW / 32)));
          umma<kTF32, kPair>(dacc, smem_desc_kmajor<kSW>(a0 + ka), smem_desc_kmajor<kSW>(b0 + kbo), kIdesc, acc);
          if constexpr (!kF8 && form_has_b2(kForm)) {
            const uint32_t b1 = a0 + kOffB2;            // Bl
            umma<kTF32, kPair>(dacc, smem_desc_kmajor<kSW>(a0 + ka), smem_desc_kmajor<kSW>(b1 + kbo), kIdesc, 1u);
            if constexpr (form_has_a2(kForm)) {
              const uint32_t a1 = a0 + kOffA2;          // Al
              umma<kTF32, kPair>(dacc, smem_desc_kmajor<kSW>(a1 + ka), smem_desc_kmajor<kSW>(b0 + kbo), kIdesc, 1u);
              if constexpr (kForm == kSplit4)
                umma<kTF32, kPair>(dacc, smem_desc_kmajor<kSW>(a1 + ka), smem_desc_kmajor<kSW>(b1 + kbo), kIdesc, 1u);
            }
          }
        }
        if constexpr (kF8) {
          // the low products: E4M3 A8 x Bl8 over the same K elements, after the stage's FP16 products
          const uint32_t a8 = a0 + kOffA2, b8 = a0 + kOffB2;
#pragma unroll
          for (int k = 0; k < kKSteps2; ++k) {
            const uint32_t ka = (uint32_t)((k / (kSW2 / 32)) * kTileM * kSW2 + 32 * (k % (kSW2 / 32)));
            const uint32_t kbo = (uint32_t)((k / (kSW2 / 32)) * kBRows * kSW2 + 32 * (k % (kSW2 / 32)));
            umma_f8<kPair>(dacc, smem_desc_kmajor<kSW2>(a8 + ka), smem_desc_kmajor<kSW2>(b8 + kbo), kIdesc8, 1u);
          }
        }
        // the stage is reusable once these MMAs have read it (in both CTAs of a pair)
        umma_commit<kPair>(smem_u32(&empty[s]));
        if constexpr (kPair) umma_commit<kPair>(empty_peer + (uint32_t)s * 8u);
        if (kin == drain_kb - 1 || kb == num_kb - 1) {
          umma_commit<kPair>(smem_u32(&acc_full[ab]));
          if constexpr (kPair) umma_commit<kPair>(accf_peer + (uint32_t)ab * 8u);
        }
      }
      // every MMA issued above has completed before the TMEM (and a pair's shared memory) is
      // released, also when a wait gave up and the loop stopped early
      umma_commit<kPair>(smem_u32(mma_done));
      mbar_wait_teardown(mma_done, 0u);
    }
  } else {
    // ---------------- drain warps 0-7, then the epilogue
    const int quad = warp & 3, half = warp >> 2;
    const uint32_t tlane = (uint32_t)(quad * 32) << 16;
    uint32_t acce_leader = 0;
    if constexpr (kPair) acce_leader = cluster_addr(acc_empty, 0);
    float sum[kHalfGroups][32];
#pragma unroll
    for (int g = 0; g < kHalfGroups; ++g)
#pragma unroll
      for (int j = 0; j < 32; ++j) sum[g][j] = 0.0f;
    int go = 1;
    for (int ch = 0; ch < nchunks; ++ch) {
      const int ab = ch & 1;
      // one lane polls; the others wait in the shuffle (warp-uniform: tcgen05.ld is .sync.aligned)
      if (lane == 0) go = mbar_wait_sleep(&acc_full[ab], (uint32_t)(ch >> 1) & 1u, 3, abort_flag) && !*abort_flag;
      go = __shfl_sync(0xffffffffu, go, 0);
      __syncwarp();
      if (!go) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t taddr = tmem_base + tlane + (uint32_t)ab * kAccCols;
#pragma unroll
      for (int g = 0; g < kHalfGroups; ++g) {
        const int grp = 2 * g + half;
        if (grp < kGroups) {  // within the allocation: kAccCols >= BN rounded up to 32
          uint32_t v[32];
          tmem_ld32(taddr + (uint32_t)(grp * 32), v);
#pragma unroll
          for (int j = 0; j < 32; ++j) sum[g][j] += __uint_as_float(v[j]);
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) {
        if constexpr (kPair) mbar_arrive_cluster(acce_leader + (uint32_t)ab * 8u);
        else mbar_arrive(&acc_empty[ab]);
      }
    }
    if (go && (int64_t)row_block * kTileM < nrows) {
      const int64_t r = (int64_t)row_block * kTileM + quad * 32 + lane;
#pragma unroll
      for (int g = 0; g < kHalfGroups; ++g) {
        const int grp = 2 * g + half;
        if (grp >= kGroups) continue;
        const int64_t cbase = (int64_t)tc.bn * BN + grp * 32;
        const int lim = BN - grp * 32 < 32 ? BN - grp * 32 : 32;  // a width of 16 (mod 32) ends on half a group
        if (mode == 1) {
          if (colmap) {  // column j of the tile goes to row colmap[j] of D (skipped when negative)
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              if (j >= lim) break;
              const int32_t dc = __ldg(colmap + cbase + j);
              if (dc >= 0) D[(int64_t)dc * ldd + r] = sum[g][j] * scale;
            }
          } else {
#pragma unroll
            for (int j = 0; j < 32; ++j)
              if (j < lim) D[(cbase + j) * ldd + r] = sum[g][j] * scale;
          }
        } else {
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int64_t c = cbase + j;
            if (c <= r) {
              const float f = sum[g][j] * scale;
              D[r * ldd + c] = f;
              D[c * ldd + r] = f;
            }
          }
        }
      }
    }
  }
  __syncwarp();  // the producer and MMA warps reconverge after their single-lane loops
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  // a pair: neither CTA leaves while the leader's MMAs may still read the other's shared memory or
  // either may still arrive on the other's barriers
  if constexpr (kPair) cluster_sync();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == kMmaWarp) {
    if constexpr (kPair)
      asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(kTmemCols)
                   : "memory");
    else
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(kTmemCols)
                   : "memory");
  }
}

// ---------------------------------------------------------------- host side
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// 2D K-major map: rows x inner elements, row stride in bytes, box = slice_bytes (128: SWIZZLE_128B,
// 64: SWIZZLE_64B) x box_rows.
bool make_map_dt(CUtensorMap* m, const void* base, CUtensorMapDataType dt, int esize, uint64_t inner,
                 uint64_t rows, uint64_t row_bytes, uint32_t box_rows, int slice_bytes) {
  auto fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[2] = {inner, rows};
  const cuuint64_t strides[1] = {row_bytes};
  const cuuint32_t box[2] = {(cuuint32_t)(slice_bytes / esize), box_rows};
  const cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(m, dt, 2, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  slice_bytes == 64 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

bool make_map(CUtensorMap* m, const void* base, bool f32, uint64_t inner, uint64_t rows,
              uint64_t row_bytes, uint32_t box_rows, int slice_bytes = kRowBytes) {
  return make_map_dt(m, base, f32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, f32 ? 4 : 2,
                     inner, rows, row_bytes, box_rows, slice_bytes);
}

template <int BN, int S, int kForm, bool kPair, int RB = kRowBytes>
constexpr size_t smem_bytes() {
  const size_t brows = kPair ? BN / 2 : BN, rb2 = form_rb2(kForm, RB);
  return (size_t)S * ((size_t)kTileM * RB + brows * RB + (form_has_a2(kForm) ? (size_t)kTileM * rb2 : 0) +
                      (form_has_b2(kForm) ? brows * rb2 : 0)) +
         1024 + 256;
}

// Launches ntiles output tiles (ntiles CTAs, or ntiles 2-CTA clusters for a CTA pair).
template <bool kTF32, int BN, int S, int kForm, bool kPair = false, int RB = kRowBytes>
cudaError_t launch(const CUtensorMap& a, const CUtensorMap& b, const CUtensorMap& a2,
                   const CUtensorMap& b2, const TileCoord* tiles, int ntiles, int num_kb, int drain_kb,
                   float* D, int64_t ldd, float scale, int mode, cudaStream_t s, int64_t nrows,
                   const int32_t* colmap = nullptr) {
  auto k = tc_gemm_kernel<kTF32, BN, S, kForm, kPair, RB>;
  constexpr size_t sm = smem_bytes<BN, S, kForm, kPair, RB>();
  static_assert(sm <= 232448, "stage ring exceeds the 227 KB of dynamic shared memory per CTA");
  static_assert(2 * S + 5 <= 31, "barriers, TMEM slot and abort flag fit the 256-byte tail");
  if (drain_kb < 1) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)ntiles * (kPair ? 2u : 1u));
  cfg.blockDim = dim3(kGemmThreads);
  cfg.dynamicSmemBytes = sm;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = kPair ? 1 : 0;
  e = cudaLaunchKernelEx(&cfg, k, a, b, a2, b2, tiles, num_kb, drain_kb, D, ldd, scale, mode, nrows, colmap);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

// Tile table of one GEMM call site: built on the host, staged in pinned memory and copied up
// asynchronously (the launching stream drains before the table is rebuilt: every caller
// synchronises on its result before the next call).
struct TileCache {
  std::vector<TileCoord> host;
  TileCoord* dev = nullptr;
  TileCoord* pinned = nullptr;
  size_t cap = 0;
};

// A table grows geometrically from 64 Ki tiles (512 KB): cudaFree waits for the whole device, so a
// launch should almost never find its table too small.
cudaError_t upload_tiles(TileCache& tc, cudaStream_t s) {
  if (tc.host.size() > tc.cap) {
    if (tc.dev) cudaFree(tc.dev);
    if (tc.pinned) cudaFreeHost(tc.pinned);
    tc.dev = nullptr;
    tc.pinned = nullptr;
    const size_t cap = std::max<size_t>({tc.host.size(), 2 * tc.cap, (size_t)1 << 16});
    tc.cap = 0;
    cudaError_t e = cudaMalloc(&tc.dev, cap * sizeof(TileCoord));
    if (e == cudaSuccess) e = cudaHostAlloc(&tc.pinned, cap * sizeof(TileCoord), cudaHostAllocDefault);
    if (e != cudaSuccess) {
      if (tc.dev) cudaFree(tc.dev);
      tc.dev = nullptr;
      tc.pinned = nullptr;
      return e;
    }
    tc.cap = cap;
  }
  std::memcpy(tc.pinned, tc.host.data(), tc.host.size() * sizeof(TileCoord));
  return cudaMemcpyAsync(tc.dev, tc.pinned, tc.host.size() * sizeof(TileCoord), cudaMemcpyHostToDevice, s);
}

cudaError_t check_error_flag(cudaStream_t s) {
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return e;
  int h = 0;
  e = cudaMemcpyFromSymbol(&h, g_tc_error, sizeof(int));
  if (e != cudaSuccess) return e;
  if (h != 0) {
    const int zero = 0;
    cudaMemcpyToSymbol(g_tc_error, &zero, sizeof(int));
    return cudaErrorLaunchTimeout;
  }
  return cudaSuccess;
}

}  // namespace

__global__ void split_tf32_kernel(const float* __restrict__ x, float* __restrict__ hi,
                                  float* __restrict__ lo, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float v = x[i];
  // round to nearest at bit 13 (ties away from zero in magnitude), keep 10 explicit mantissa bits
  const uint32_t u = __float_as_uint(v);
  const float h = isfinite(v) ? __uint_as_float((u + 0x1000u) & 0xFFFFE000u) : v;
  // v - h is exact in FP32: |v - h| <= 2^-11 |v| and both share v's exponent range
  hi[i] = h;
  lo[i] = isfinite(v) ? v - h : 0.0f;
}


void launch_split_tf32(const float* x, float* hi, float* lo, int64_t n, cudaStream_t s) {
  if (n == 0) return;
  split_tf32_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(x, hi, lo, n);
}

// x (+ x2) = hi + lo with hi = bf16_rn(x), lo = bf16_rn(x - hi): 16 significant bits in all.
// x - hi is exact in FP32 (|x - hi| <= half a bf16 ulp of x).  Two elements per thread.
__global__ void split_bf16_kernel(const float* __restrict__ x, const float* __restrict__ x2,
                                  __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo, int64_t n) {
  const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * 2;
  if (i >= n) return;
  float v[2] = {x[i], i + 1 < n ? x[i + 1] : 0.0f};
  if (x2) {
    v[0] += x2[i];
    if (i + 1 < n) v[1] += x2[i + 1];
  }
  __nv_bfloat16 h[2], l[2];
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    h[j] = __float2bfloat16_rn(v[j]);
    l[j] = isfinite(v[j]) ? __float2bfloat16_rn(v[j] - __bfloat162float(h[j])) : __float2bfloat16_rn(0.0f);
  }
  if (i + 1 < n) {
    *reinterpret_cast<__nv_bfloat162*>(hi + i) = __halves2bfloat162(h[0], h[1]);
    *reinterpret_cast<__nv_bfloat162*>(lo + i) = __halves2bfloat162(l[0], l[1]);
  } else {
    hi[i] = h[0];
    lo[i] = l[0];
  }
}

// Compact BF16 halves of selected columns: column j of (hi, lo) is column cols[j] of x (np rows
// each), or zeros when cols[j] < 0 (padding up to the GRM.V tile width).
__global__ void split_bf16_gather_kernel(const float* __restrict__ x, int64_t np, const int32_t* __restrict__ cols,
                                         __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo) {
  const int64_t j = blockIdx.y;
  const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * 4;
  if (i >= np) return;  // np is a multiple of 128
  const int32_t c = cols[j];
  float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
  if (c >= 0) v = *reinterpret_cast<const float4*>(x + (int64_t)c * np + i);
  const float a[4] = {v.x, v.y, v.z, v.w};
  __nv_bfloat16 h[4], l[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    h[k] = __float2bfloat16_rn(a[k]);
    l[k] = isfinite(a[k]) ? __float2bfloat16_rn(a[k] - __bfloat162float(h[k])) : __float2bfloat16_rn(0.0f);
  }
  __nv_bfloat162* ho = reinterpret_cast<__nv_bfloat162*>(hi + j * np + i);
  __nv_bfloat162* lw = reinterpret_cast<__nv_bfloat162*>(lo + j * np + i);
  ho[0] = __halves2bfloat162(h[0], h[1]);
  ho[1] = __halves2bfloat162(h[2], h[3]);
  lw[0] = __halves2bfloat162(l[0], l[1]);
  lw[1] = __halves2bfloat162(l[2], l[3]);
}

void launch_split_bf16_gather(const float* x, int64_t np, const int32_t* cols, int64_t ncols, void* hi,
                              void* lo, cudaStream_t s) {
  if (ncols == 0) return;
  dim3 grid((unsigned)((np / 4 + 255) / 256), (unsigned)ncols);
  split_bf16_gather_kernel<<<grid, 256, 0, s>>>(x, np, cols, static_cast<__nv_bfloat16*>(hi),
                                                static_cast<__nv_bfloat16*>(lo));
}

void launch_split_bf16(const float* x, const float* x2, void* hi, void* lo, int64_t n, cudaStream_t s) {
  if (n == 0) return;
  const int64_t threads = (n + 1) / 2;
  split_bf16_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(
      x, x2, static_cast<__nv_bfloat16*>(hi), static_cast<__nv_bfloat16*>(lo), n);
}


cudaError_t tc_wait_selftest(double budget_ms, int* waited_out, cudaStream_t s) {
  int* d = nullptr;
  cudaError_t e = cudaMallocAsync(&d, sizeof(int), s);
  if (e != cudaSuccess) return e;
  wait_selftest_kernel<<<1, 32, 0, s>>>((unsigned long long)(budget_ms * 1e6), d);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(waited_out, d, sizeof(int), cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(d, s);
  if (e != cudaSuccess) return e;
  return check_error_flag(s);  // cudaErrorLaunchTimeout when the wait ran out (flag then cleared)
}

bool tc_available() {
  int dev = 0, major = 0, minor = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  return major == 10 && minor == 3 && encode_fn() != nullptr;
}

// Shape options of the tcgen05 GEMMs (process-wide; saigegpu.tune sets them from timings).
static int g_opt[kTcOptions] = {
    1,    // kTcSyrkPair: SYRK tiles on CTA pairs (cta_group::2, 256 x 256)
    0,    // kTcGrmvPair: split GRM.V tiles on CTA pairs (256 x BN)
    512,  // kTcDrainBytes: bytes of K per row one TMEM accumulator takes before it is drained
    8,    // kTcSyrkGroup: row tiles per raster group of the SYRK
    0,    // kTcGrmvSlice: K slice bytes of the split-BF16 GRM.V (0: by width, 64 or 128)
    2,    // kTcSubsetPair: subset-exact genotype GEMMs on CTA pairs (2: above 160 columns)
    256,  // kTcSubsetSlice: their K-stage bytes (0: 128 up to 160 columns, else 64; or 64 / 128 / 256 / 512)
};

bool tc_set_option(int opt, int value) {
  if (opt < 0 || opt >= kTcOptions) return false;
  switch (opt) {
    case kTcSyrkPair:
    case kTcGrmvPair:
      if (value != 0 && value != 1) return false;
      break;
    case kTcSubsetPair:
      if (value < 0 || value > 2) return false;
      break;
    case kTcDrainBytes:  // whole 128-byte stages, at most 4 KB (the bias grows with the length)
      if (value < 128 || value > 4096 || value % 128 != 0) return false;
      break;
    case kTcSyrkGroup:
      if (value < 1 || value > 4096) return false;
      break;
    case kTcGrmvSlice:
      if (value != 0 && value != 64 && value != 128) return false;
      break;
    case kTcSubsetSlice:
      if (value != 0 && value != 64 && value != 128 && value != 256 && value != 512) return false;
      break;
  }
  g_opt[opt] = value;
  return true;
}

int tc_get_option(int opt) { return opt >= 0 && opt < kTcOptions ? g_opt[opt] : -1; }

// Per-launch-width choices of the split-BF16 GRM.V (the tuner's table): the first bucket whose
// max_cols covers a launch's columns gives its CTA-pair and K-slice choice; wider launches, or no
// table, use the process-wide options.
struct GrmvChoice {
  int64_t max_cols;
  int pair, slice;
};
static std::vector<GrmvChoice> g_plan;

bool tc_set_grmv_plan(const int32_t* max_cols, const int32_t* pair, const int32_t* slice, int n) {
  std::vector<GrmvChoice> plan;
  for (int i = 0; i < n; ++i) {
    if (max_cols[i] <= 0 || (i > 0 && max_cols[i] <= max_cols[i - 1])) return false;
    if ((pair[i] != 0 && pair[i] != 1) || (slice[i] != 0 && slice[i] != 64 && slice[i] != 128)) return false;
    plan.push_back(GrmvChoice{max_cols[i], pair[i], slice[i]});
  }
  g_plan.swap(plan);
  return true;
}

int tc_get_grmv_plan(int32_t* max_cols, int32_t* pair, int32_t* slice, int cap) {
  const int n = (int)g_plan.size();
  for (int i = 0; i < n && i < cap; ++i) {
    max_cols[i] = (int32_t)g_plan[i].max_cols;
    pair[i] = g_plan[i].pair;
    slice[i] = g_plan[i].slice;
  }
  return n;
}

static GrmvChoice grmv_choice(int64_t ncols) {
  for (const GrmvChoice& b : g_plan)
    if (ncols <= b.max_cols) return b;
  return GrmvChoice{0, g_opt[kTcGrmvPair], g_opt[kTcGrmvSlice]};
}

// The same kind of table for the subset-exact engine's genotype GEMMs.
static std::vector<GrmvChoice> g_subset_plan;

bool tc_set_subset_plan(const int32_t* max_cols, const int32_t* pair, const int32_t* slice, int n) {
  std::vector<GrmvChoice> plan;
  for (int i = 0; i < n; ++i) {
    if (max_cols[i] <= 0 || (i > 0 && max_cols[i] <= max_cols[i - 1])) return false;
    if ((pair[i] != 0 && pair[i] != 1) ||
        (slice[i] != 64 && slice[i] != 128 && slice[i] != 256 && slice[i] != 512))
      return false;
    plan.push_back(GrmvChoice{max_cols[i], pair[i], slice[i]});
  }
  g_subset_plan.swap(plan);
  return true;
}

int tc_get_subset_plan(int32_t* max_cols, int32_t* pair, int32_t* slice, int cap) {
  const int n = (int)g_subset_plan.size();
  for (int i = 0; i < n && i < cap; ++i) {
    max_cols[i] = (int32_t)g_subset_plan[i].max_cols;
    pair[i] = g_subset_plan[i].pair;
    slice[i] = g_subset_plan[i].slice;
  }
  return n;
}

static int drain_stages(int rb) { return g_opt[kTcDrainBytes] / rb > 0 ? g_opt[kTcDrainBytes] / rb : 1; }

// Lower-triangle tiles of the SYRK in raster groups: ``group`` consecutive row tiles (of ``unit``
// 128-row blocks each) sweep the column blocks together, column block by column block, so that the
// tiles resident at one time share a few row panels and a few column panels of Z in L2 instead of
// one row panel and a whole row of column panels.  Column block bn (BN wide) of a row tile is
// kept when it starts at or before the tile's last row; tiles above a row block's diagonal store
// nothing, and a trailing row block past np loads zeros and stores nothing.
static void syrk_tiles(std::vector<TileCoord>& out, int64_t np, int BN, int unit, int group) {
  out.clear();
  const int64_t nbm = np / kTileM;
  const int64_t nrt = (nbm + unit - 1) / unit;
  for (int64_t g0 = 0; g0 < nrt; g0 += group) {
    const int64_t g1 = g0 + group < nrt ? g0 + group : nrt;
    for (int64_t bn = 0;; ++bn) {
      if (bn * BN >= np) break;
      bool any = false;
      for (int64_t rt = g0; rt < g1; ++rt) {
        const int64_t last_row = (rt * unit + unit) * kTileM - 1;
        if (bn * BN <= last_row) {
          out.push_back(TileCoord{(int32_t)(rt * unit), (int32_t)bn});
          any = true;
        }
      }
      if (!any) break;
    }
  }
}

cudaError_t tc_syrk_bf16(const void* Zhi, const void* Zlo, int64_t np, int64_t mp, float* K,
                         float scale, cudaStream_t s) {
  constexpr int BN = 256;
  if (np % kTileM != 0 || mp % 64 != 0) return cudaErrorInvalidValue;
  const bool pair = g_opt[kTcSyrkPair] != 0;
  // 128-byte K slices: 4 stages of 48 KB per CTA (2 for the split build), or on a CTA pair 6
  // stages of 32 KB (3 for the split build)
  constexpr int RB = 128;
  CUtensorMap a, b, a2, b2;
  const uint64_t rb = (uint64_t)mp * 2;
  const uint32_t brows = (uint32_t)(pair ? BN / 2 : BN);  // a pair's CTAs load half of B each
  if (!make_map(&a, Zhi, false, mp, np, rb, kTileM, RB) || !make_map(&b, Zhi, false, mp, np, rb, brows, RB))
    return cudaErrorInvalidValue;
  a2 = a;
  b2 = b;
  if (Zlo && (!make_map(&a2, Zlo, false, mp, np, rb, kTileM, RB) || !make_map(&b2, Zlo, false, mp, np, rb, brows, RB)))
    return cudaErrorInvalidValue;
  static TileCache cache;
  syrk_tiles(cache.host, np, BN, pair ? 2 : 1, g_opt[kTcSyrkGroup]);
  cudaError_t e = upload_tiles(cache, s);
  if (e != cudaSuccess) return e;
  const int num_kb = (int)(mp / (RB / 2));
  const int nt = (int)cache.host.size();
  const int dk = drain_stages(RB);
  if (Zlo) {
    // all four products: the residuals Zl of a marker take only three values (one per genotype),
    // so the Zl Zl' term does not average out over markers (dropping it left the off-diagonal
    // entries ~7e-7 off at M = 150k, against ~2e-9 with it)
    e = pair ? launch<false, BN, 3, kSplit4, true, RB>(a, b, a2, b2, cache.dev, nt, num_kb, dk, K, np, scale, 2, s, np)
             : launch<false, BN, 2, kSplit4, false, RB>(a, b, a2, b2, cache.dev, nt, num_kb, dk, K, np, scale, 2, s, np);
  } else {
    e = pair ? launch<false, BN, 6, kOne, true, RB>(a, b, a2, b2, cache.dev, nt, num_kb, dk, K, np, scale, 2, s, np)
             : launch<false, BN, 4, kOne, false, RB>(a, b, a2, b2, cache.dev, nt, num_kb, dk, K, np, scale, 2, s, np);
  }
  if (e != cudaSuccess) return e;
  return check_error_flag(s);
}

// Column-tile widths of the GRM.V.  The split variants also come in 96..224 so that a column
// count rarely needs padding to the next power of two.
static const std::vector<int> kSplitWidths = {256, 224, 192, 160, 128, 96, 64, 32};
// split-BF16 also has the widths that are odd multiples of 16 (clusters of at most 2 CTAs)
static const std::vector<int> kBf16Widths = {256, 224, 208, 192, 176, 160, 144, 128, 112, 96, 80, 64, 48, 32};
static const std::vector<int> kPlainWidths = {256, 128, 64, 32};

static const std::vector<int>& tile_widths(int set) {
  return set == kTilesSplitBF16 ? kBf16Widths
         : (set == kTilesSplitTF32 || set == kTilesSplitB) ? kSplitWidths
                                                           : kPlainWidths;
}

// Column-tile width for ncols columns: the widest tile that divides ncols (wider tiles re-read
// the K strip fewer times).  A lone 256-wide block is split in two for more CTAs per wave.
int tc_gemm_tile_n(int64_t ncols, int set) {
  for (int w : tile_widths(set)) {
    if (w == 256 && ncols < 512 && set == kTilesPlain) continue;
    if (ncols % w == 0) return w;
  }
  return set == kTilesSplitBF16 ? 16 : 32;
}

// CTA pairs for a subset-exact genotype GEMM over ncols columns: measured at N = 100k, M = 150k,
// 256-byte K stages, pairs took 512 columns from 49.7 to 32.8 ms and 1024 from 89.4 to 61.8 ms,
// and were 5-12% slower up to 128 columns, where the launch streams G from HBM.
static bool subset_pair(int64_t ncols) {
  for (const GrmvChoice& b : g_subset_plan)
    if (ncols <= b.max_cols) return b.pair != 0;
  return g_opt[kTcSubsetPair] == 2 ? ncols > 160 : g_opt[kTcSubsetPair] != 0;
}

static int subset_slice(int64_t ncols) {
  for (const GrmvChoice& b : g_subset_plan)
    if (ncols <= b.max_cols) return b.slice;
  return g_opt[kTcSubsetSlice] != 0 ? g_opt[kTcSubsetSlice] : (ncols <= 160 ? 128 : 64);
}

// 256- and 512-byte stages exist for the tile widths whose stage (128 A rows and two halves of the
// B rows, RB bytes each) leaves room for at least two stages; other widths fall back to the next
// smaller stage that has a table.
static int splitb_stage_bytes(int RB, int BN, bool pair) {
  if (RB == 512 && !(BN == 32 || (pair && BN == 64))) RB = 256;
  if (RB == 256 && !(pair || BN <= 160)) RB = 128;
  return RB;
}

// Columns one GRM.V launch covers for ncols32 (a multiple of 16) live columns, padded so that the
// modelled cost is lowest, capped at cap columns.  Cost model (L2->SM bytes of one pass, which
// bounds these kernels, over the fraction of the last wave of 1-tile-per-SM(-pair) tiles that is
// busy): padded * (A bytes per stage / BN + B bytes per stage per column) / wave_efficiency; a CTA
// pair loads half of the B tile per SM and fills num_sms / 2 tile slots per wave.
int64_t tc_grmv_padded_cols(int64_t ncols32, int64_t cap, int64_t np, int set, int num_sms) {
  double best = 1e300;
  int64_t best_cols = ncols32;
  for (int w : tile_widths(set)) {
    const int64_t padded = (ncols32 + w - 1) / w * w;
    if (padded > cap) continue;
    const bool pair = (set == kTilesSplitBF16 && grmv_choice(padded).pair != 0) ||
                      (set == kTilesSplitB && subset_pair(padded));
    const int64_t nrt = pair ? (np / kTileM + 1) / 2 : np / kTileM;
    const int64_t slots = pair ? num_sms / 2 : num_sms;
    const int bn = tc_gemm_tile_n(padded, set);
    const int64_t tiles = nrt * (padded / bn);
    const int64_t waves = (tiles + slots - 1) / slots;
    const double eff = (double)tiles / (double)(waves * slots);
    const double cost = (double)padded * ((double)kATileBytes / bn + (double)kRowBytes / (pair ? 2 : 1)) / eff;
    if (cost < best) {
      best = cost;
      best_cols = padded;
    }
  }
  return best_cols;
}

// K slice bytes of a split GRM.V launch over ncols columns: 128 for split-TF32; for split-BF16, 64
// (twice the stages: measured 10% faster at 256 columns, 8-12% from there up) once the launch is
// bound by the tensor pipe, and 128 while it streams K from HBM (at most 160 columns: half as many,
// larger stages, measured 3% faster at 128 columns); kTcGrmvSlice overrides the split-BF16 choice.
static int grmv_slice_bytes(bool tf32, int64_t ncols) {
  if (tf32) return 128;
  const int slice = grmv_choice(ncols).slice;
  if (slice != 0) return slice;
  return ncols <= 160 ? 128 : 64;
}

template <bool kTF32, int BN, int S, bool kPair, int RB>
static cudaError_t launch_grmv_split(const CUtensorMap& a, const CUtensorMap& b, const CUtensorMap& a2,
                                     const CUtensorMap& b2, const TileCoord* tiles, int nt, int num_kb,
                                     float* Y, int64_t np, cudaStream_t s, const int32_t* colmap) {
  return launch<kTF32, BN, S, kSplit3, kPair, RB>(a, b, a2, b2, tiles, nt, num_kb, drain_stages(RB), Y, np, 1.0f,
                                               1, s, np, colmap);
}

// Split GRM.V over every tile width, with as many pipeline stages as the 227 KB of shared memory
// hold at that width (per CTA: two halves of 128 K rows plus BN -- or BN / 2 on a CTA pair -- P rows).
template <bool kTF32>
static cudaError_t grmv_split_dispatch(int BN, bool pair, int RB, const CUtensorMap& a, const CUtensorMap& b,
                                       const CUtensorMap& a2, const CUtensorMap& b2, const TileCoord* tiles,
                                       int nt, int num_kb, float* Y, int64_t np, cudaStream_t s,
                                       const int32_t* colmap = nullptr) {
#define SG_GRMV_ARGS a, b, a2, b2, tiles, nt, num_kb, Y, np, s, colmap
#define SG_GRMV_CASE(BNv, Sv, RBv) \
  case BNv:                        \
    return launch_grmv_split<kTF32, BNv, Sv, false, RBv>(SG_GRMV_ARGS);
#define SG_GRMV_PAIR(BNv, Sv, RBv) \
  case BNv:                        \
    return launch_grmv_split<kTF32, BNv, Sv, true, RBv>(SG_GRMV_ARGS);
  if constexpr (!kTF32) {
    if (pair && RB == 64) {
      switch (BN) {
        SG_GRMV_PAIR(256, 7, 64)
        SG_GRMV_PAIR(224, 7, 64)
        SG_GRMV_PAIR(208, 7, 64)
        SG_GRMV_PAIR(192, 8, 64)
        SG_GRMV_PAIR(176, 8, 64)
        SG_GRMV_PAIR(160, 8, 64)
        SG_GRMV_PAIR(144, 9, 64)
        SG_GRMV_PAIR(128, 9, 64)
        SG_GRMV_PAIR(112, 9, 64)
        SG_GRMV_PAIR(96, 10, 64)
        SG_GRMV_PAIR(80, 10, 64)
        SG_GRMV_PAIR(64, 11, 64)
        SG_GRMV_PAIR(48, 11, 64)
        SG_GRMV_PAIR(32, 12, 64)
        default:
          return cudaErrorInvalidValue;
      }
    }
    if (pair) {
      switch (BN) {
        SG_GRMV_PAIR(256, 3, 128)
        SG_GRMV_PAIR(224, 3, 128)
        SG_GRMV_PAIR(208, 3, 128)
        SG_GRMV_PAIR(192, 4, 128)
        SG_GRMV_PAIR(176, 4, 128)
        SG_GRMV_PAIR(160, 4, 128)
        SG_GRMV_PAIR(144, 4, 128)
        SG_GRMV_PAIR(128, 4, 128)
        SG_GRMV_PAIR(112, 4, 128)
        SG_GRMV_PAIR(96, 5, 128)
        SG_GRMV_PAIR(80, 5, 128)
        SG_GRMV_PAIR(64, 5, 128)
        SG_GRMV_PAIR(48, 5, 128)
        SG_GRMV_PAIR(32, 6, 128)
        default:
          return cudaErrorInvalidValue;
      }
    }
    if (RB == 64) {
      // (8 KB + BN x 64 B) x 2 halves per stage, as many stages as fit
      switch (BN) {
        SG_GRMV_CASE(256, 4, 64)
        SG_GRMV_CASE(224, 5, 64)
        SG_GRMV_CASE(208, 5, 64)
        SG_GRMV_CASE(192, 5, 64)
        SG_GRMV_CASE(176, 5, 64)
        SG_GRMV_CASE(160, 6, 64)
        SG_GRMV_CASE(144, 6, 64)
        SG_GRMV_CASE(128, 7, 64)
        SG_GRMV_CASE(112, 7, 64)
        SG_GRMV_CASE(96, 8, 64)
        SG_GRMV_CASE(80, 8, 64)
        SG_GRMV_CASE(64, 9, 64)
        SG_GRMV_CASE(48, 10, 64)
        SG_GRMV_CASE(32, 11, 64)
        default:
          return cudaErrorInvalidValue;
      }
    }
    // (16 KB + BN x 128 B) x 2 halves per stage
    switch (BN) {
      SG_GRMV_CASE(256, 2, 128)
      SG_GRMV_CASE(224, 2, 128)
      SG_GRMV_CASE(208, 2, 128)
      SG_GRMV_CASE(192, 2, 128)
      SG_GRMV_CASE(176, 2, 128)
      SG_GRMV_CASE(160, 3, 128)
      SG_GRMV_CASE(144, 3, 128)
      SG_GRMV_CASE(128, 3, 128)
      SG_GRMV_CASE(112, 3, 128)
      SG_GRMV_CASE(96, 4, 128)
      SG_GRMV_CASE(80, 4, 128)
      SG_GRMV_CASE(64, 4, 128)
      SG_GRMV_CASE(48, 5, 128)
      SG_GRMV_CASE(32, 5, 128)
      default:
        return cudaErrorInvalidValue;
    }
  } else {
    (void)pair;
    // (16 KB + BN x 128 B) x 2 halves per stage
    switch (BN) {
      SG_GRMV_CASE(256, 2, 128)
      SG_GRMV_CASE(224, 2, 128)
      SG_GRMV_CASE(192, 2, 128)
      SG_GRMV_CASE(160, 3, 128)
      SG_GRMV_CASE(128, 3, 128)
      SG_GRMV_CASE(96, 4, 128)
      SG_GRMV_CASE(64, 4, 128)
      SG_GRMV_CASE(32, 5, 128)
      default:
        return cudaErrorInvalidValue;
    }
  }
#undef SG_GRMV_CASE
#undef SG_GRMV_PAIR
#undef SG_GRMV_ARGS
}

// Row tiles (one 128-row block, or two for a CTA pair; a trailing block past np loads zeros and
// stores nothing) times column blocks, column blocks fastest so that the tiles of one K row strip
// run together.
static cudaError_t grmv_tiles(TileCache& cache, int64_t np, int64_t ncols, int BN, bool pair, cudaStream_t s) {
  cache.host.clear();
  const int64_t nbm = np / kTileM;
  const int unit = pair ? 2 : 1;
  for (int64_t rt = 0; rt < (nbm + unit - 1) / unit; ++rt)
    for (int64_t bn = 0; bn < ncols / BN; ++bn) cache.host.push_back(TileCoord{(int32_t)(rt * unit), (int32_t)bn});
  return upload_tiles(cache, s);
}

cudaError_t tc_gemm_tf32(const float* K, const float* Klo, int64_t np, const float* P,
                         const float* Plo, int64_t ncols, float* Y, cudaStream_t s, bool check) {
  if (np % kTileM != 0 || ncols % 32 != 0 || ncols <= 0) return cudaErrorInvalidValue;
  const bool split = Klo != nullptr && Plo != nullptr;
  const int BN = tc_gemm_tile_n(ncols, split ? kTilesSplitTF32 : kTilesPlain);
  CUtensorMap a, b, a2, b2;
  if (!make_map(&a, K, true, np, np, (uint64_t)np * 4, kTileM) ||
      !make_map(&b, P, true, np, ncols, (uint64_t)np * 4, BN))
    return cudaErrorInvalidValue;
  a2 = a;
  b2 = b;
  if (split && (!make_map(&a2, Klo, true, np, np, (uint64_t)np * 4, kTileM) ||
                !make_map(&b2, Plo, true, np, ncols, (uint64_t)np * 4, BN)))
    return cudaErrorInvalidValue;
  static TileCache cache;
  cudaError_t e = grmv_tiles(cache, np, ncols, BN, false, s);
  if (e != cudaSuccess) return e;
  const int num_kb = (int)(np / 32);
  const int nt = (int)cache.host.size();
  const int dk = drain_stages(128);
  if (split) {
    e = grmv_split_dispatch<true>(BN, false, 128, a, b, a2, b2, cache.dev, nt, num_kb, Y, np, s);
  } else {
    switch (BN) {
      case 256: e = launch<true, 256, 3, kOne>(a, b, a, b, cache.dev, nt, num_kb, dk, Y, np, 1.0f, 1, s, np); break;
      case 128: e = launch<true, 128, 4, kOne>(a, b, a, b, cache.dev, nt, num_kb, dk, Y, np, 1.0f, 1, s, np); break;
      case 64: e = launch<true, 64, 6, kOne>(a, b, a, b, cache.dev, nt, num_kb, dk, Y, np, 1.0f, 1, s, np); break;
      default: e = launch<true, 32, 8, kOne>(a, b, a, b, cache.dev, nt, num_kb, dk, Y, np, 1.0f, 1, s, np); break;
    }
  }
  if (e != cudaSuccess) return e;
  return check ? check_error_flag(s) : cudaSuccess;
}

cudaError_t tc_gemm_bf16x3(const void* Kh, const void* Kl, int64_t np, const void* Ph, const void* Pl,
                           int64_t ncols, float* Y, cudaStream_t s, bool check, const int32_t* colmap) {
  if (np % kTileM != 0 || ncols % 16 != 0 || ncols <= 0 || !Kh || !Kl || !Ph || !Pl)
    return cudaErrorInvalidValue;
  const int BN = tc_gemm_tile_n(ncols, kTilesSplitBF16);
  const bool pair = grmv_choice(ncols).pair != 0;
  const uint32_t brows = (uint32_t)(pair ? BN / 2 : BN);
  const uint64_t rb = (uint64_t)np * 2;
  const int kSlice = grmv_slice_bytes(false, ncols);
  CUtensorMap a, b, a2, b2;
  if (!make_map(&a, Kh, false, np, np, rb, kTileM, kSlice) || !make_map(&b, Ph, false, np, ncols, rb, brows, kSlice) ||
      !make_map(&a2, Kl, false, np, np, rb, kTileM, kSlice) || !make_map(&b2, Pl, false, np, ncols, rb, brows, kSlice))
    return cudaErrorInvalidValue;
  static TileCache cache;
  cudaError_t e = grmv_tiles(cache, np, ncols, BN, pair, s);
  if (e != cudaSuccess) return e;
  const int num_kb = (int)(np / (kSlice / 2));
  e = grmv_split_dispatch<false>(BN, pair, kSlice, a, b, a2, b2, cache.dev, (int)cache.host.size(), num_kb, Y,
                                 np, s, colmap);
  if (e != cudaSuccess) return e;
  return check ? check_error_flag(s) : cudaSuccess;
}

// D = A (Bh + Bl)^T: A (rows x kdim) exact in BF16 (genotype values), B as BF16 high + low halves
// (ncols x kdim), two products per K step into the drained TMEM accumulators; D RHS-major (column j
// of the product is row j of D, leading dimension ldd).  K slices of 128 bytes by default (each
// 128-byte row segment of A is a whole DRAM burst line; measured at N = 100k, M = 150k they took
// 32-128 columns from 23-24 ms to 16 ms and, on CTA pairs, 512 columns from 54 to 36.5 ms), or
// 64 bytes (twice the stages); as many stages as fit.
cudaError_t tc_gemm_splitb(const void* A, int64_t rows, int64_t kdim, const void* Bh, const void* Bl,
                           int64_t ncols, float* D, int64_t ldd, cudaStream_t s, bool check, int site) {
  if (rows % kTileM != 0 || kdim % 64 != 0 || ncols % 32 != 0 || ncols <= 0 || !A || !Bh || !Bl || site < 0 ||
      site > 1)
    return cudaErrorInvalidValue;
  const int BN = tc_gemm_tile_n(ncols, kTilesSplitB);
  const bool pair = subset_pair(ncols);
  int RB = splitb_stage_bytes(subset_slice(ncols), BN, pair);
  while (RB > 128 && kdim % (RB / 2) != 0) RB /= 2;  // whole stages over K
  const int box = RB > 128 ? 128 : RB;  // a 256- or 512-byte stage is 2 or 4 128-byte boxes per operand
  const uint64_t rb = (uint64_t)kdim * 2;
  CUtensorMap a, b, b2;
  if (!make_map(&a, A, false, kdim, rows, rb, kTileM, box) ||
      !make_map(&b, Bh, false, kdim, ncols, rb, pair ? BN / 2 : BN, box) ||
      !make_map(&b2, Bl, false, kdim, ncols, rb, pair ? BN / 2 : BN, box))
    return cudaErrorInvalidValue;
  // one tile table per call site: the two GEMMs of an engine step are queued back to back, so the
  // second must not restage the table the first one's upload may still be reading
  static TileCache caches[2];
  TileCache& cache = caches[site];
  cudaError_t e = grmv_tiles(cache, rows, ncols, BN, pair, s);
  if (e != cudaSuccess) return e;
  const int num_kb = (int)(kdim / (RB / 2));
  const int nt = (int)cache.host.size();
  const int dk = drain_stages(RB);
#define SG_SB(BNv, Sv, Pv, RBv)                                                                              \
  case BNv:                                                                                                  \
    e = launch<false, BNv, Sv, kSplitB, Pv, RBv>(a, b, a, b2, cache.dev, nt, num_kb, dk, D, ldd, 1.0f, 1, s, \
                                                  rows);                                                    \
    break;
  // per CTA and stage: 128 A rows plus two halves of BN (BN / 2 on a CTA pair) B rows, RB bytes each
  if (RB == 512 && pair) {
    switch (BN) {
      SG_SB(64, 2, true, 512)
      SG_SB(32, 2, true, 512)
      default:
        return cudaErrorInvalidValue;
    }
  } else if (RB == 512) {
    switch (BN) {
      SG_SB(32, 2, false, 512)
      default:
        return cudaErrorInvalidValue;
    }
  } else if (RB == 256 && pair) {
    switch (BN) {
      SG_SB(256, 2, true, 256)
      SG_SB(224, 2, true, 256)
      SG_SB(192, 2, true, 256)
      SG_SB(160, 3, true, 256)
      SG_SB(128, 3, true, 256)
      SG_SB(96, 4, true, 256)
      SG_SB(64, 4, true, 256)
      SG_SB(32, 5, true, 256)
      default:
        return cudaErrorInvalidValue;
    }
  } else if (RB == 256) {
    switch (BN) {
      SG_SB(160, 2, false, 256)
      SG_SB(128, 2, false, 256)
      SG_SB(96, 2, false, 256)
      SG_SB(64, 3, false, 256)
      SG_SB(32, 4, false, 256)
      default:
        return cudaErrorInvalidValue;
    }
  } else if (RB == 128 && pair) {
    switch (BN) {
      SG_SB(256, 4, true, 128)
      SG_SB(224, 4, true, 128)
      SG_SB(192, 5, true, 128)
      SG_SB(160, 6, true, 128)
      SG_SB(128, 7, true, 128)
      SG_SB(96, 8, true, 128)
      SG_SB(64, 9, true, 128)
      SG_SB(32, 11, true, 128)
      default:
        return cudaErrorInvalidValue;
    }
  } else if (RB == 128) {
    switch (BN) {
      SG_SB(256, 2, false, 128)
      SG_SB(224, 3, false, 128)
      SG_SB(192, 3, false, 128)
      SG_SB(160, 4, false, 128)
      SG_SB(128, 4, false, 128)
      SG_SB(96, 5, false, 128)
      SG_SB(64, 7, false, 128)
      SG_SB(32, 9, false, 128)
      default:
        return cudaErrorInvalidValue;
    }
  } else if (pair) {
    switch (BN) {
      SG_SB(256, 9, true, 64)
      SG_SB(224, 10, true, 64)
      SG_SB(192, 11, true, 64)
      SG_SB(160, 12, true, 64)
      SG_SB(128, 12, true, 64)
      SG_SB(96, 12, true, 64)
      SG_SB(64, 12, true, 64)
      SG_SB(32, 12, true, 64)
      default:
        return cudaErrorInvalidValue;
    }
  } else {
    switch (BN) {
      SG_SB(256, 5, false, 64)
      SG_SB(224, 6, false, 64)
      SG_SB(192, 7, false, 64)
      SG_SB(160, 8, false, 64)
      SG_SB(128, 9, false, 64)
      SG_SB(96, 11, false, 64)
      SG_SB(64, 12, false, 64)
      SG_SB(32, 12, false, 64)
      default:
        return cudaErrorInvalidValue;
    }
  }
#undef SG_SB
  if (e != cudaSuccess) return e;
  return check ? check_error_flag(s) : cudaSuccess;
}

// The same GEMM with the high halves in FP16 and the low halves in E4M3: D = A Bh + A8 Bl8, A (FP16)
// and A8 (E4M3) the same exact values, K stages of 256 bytes of A (128 elements; the E4M3 operands
// take one 128-byte box per row and stage).  The low products run at twice the FP16 rate, so a
// stage costs three quarters of the two FP16 (or BF16) products' time.  Tiles of more than 160
// columns run on CTA pairs (a single CTA has room for one such stage only).
cudaError_t tc_gemm_splitb8(const void* A, const void* A8, int64_t rows, int64_t kdim, const void* Bh,
                            const void* Bl8, int64_t ncols, float* D, int64_t ldd, cudaStream_t s, bool check,
                            int site) {
  if (rows % kTileM != 0 || kdim % 128 != 0 || ncols % 32 != 0 || ncols <= 0 || !A || !A8 || !Bh || !Bl8 ||
      site < 0 || site > 1)
    return cudaErrorInvalidValue;
  const int BN = tc_gemm_tile_n(ncols, kTilesSplitB);
  const bool pair = subset_pair(ncols) || BN > 160;
  const int brows = pair ? BN / 2 : BN;
  CUtensorMap a, b, a8, b8;
  if (!make_map_dt(&a, A, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, kdim, rows, (uint64_t)kdim * 2, kTileM, 128) ||
      !make_map_dt(&b, Bh, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, kdim, ncols, (uint64_t)kdim * 2, brows, 128) ||
      !make_map_dt(&a8, A8, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, kdim, rows, (uint64_t)kdim, kTileM, 128) ||
      !make_map_dt(&b8, Bl8, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, kdim, ncols, (uint64_t)kdim, brows, 128))
    return cudaErrorInvalidValue;
  static TileCache caches[2];
  TileCache& cache = caches[site];
  cudaError_t e = grmv_tiles(cache, rows, ncols, BN, pair, s);
  if (e != cudaSuccess) return e;
  const int num_kb = (int)(kdim / 128);
  const int nt = (int)cache.host.size();
  const int dk = drain_stages(256);
#define SG_SB8(BNv, Sv, Pv)                                                                                  \
  case BNv:                                                                                                  \
    e = launch<false, BNv, Sv, kSplitB8, Pv, 256>(a, b, a8, b8, cache.dev, nt, num_kb, dk, D, ldd, 1.0f, 1, s, \
                                                  rows);                                                    \
    break;
  // per CTA and stage: 128 A rows (256 B FP16 + 128 B E4M3) and BN (BN / 2 on a pair) B rows alike
  if (pair) {
    switch (BN) {
      SG_SB8(256, 2, true)
      SG_SB8(224, 2, true)
      SG_SB8(192, 2, true)
      SG_SB8(160, 2, true)
      SG_SB8(128, 3, true)
      SG_SB8(96, 3, true)
      SG_SB8(64, 3, true)
      SG_SB8(32, 4, true)
      default:
        return cudaErrorInvalidValue;
    }
  } else {
    switch (BN) {
      SG_SB8(160, 2, false)
      SG_SB8(128, 2, false)
      SG_SB8(96, 2, false)
      SG_SB8(64, 3, false)
      SG_SB8(32, 3, false)
      default:
        return cudaErrorInvalidValue;
    }
  }
#undef SG_SB8
  if (e != cudaSuccess) return e;
  return check ? check_error_flag(s) : cudaSuccess;
}

cudaError_t tc_check_error(cudaStream_t s) { return check_error_flag(s); }

// ---------------------------------------------------------------- GRM.V that allocates nothing
//
// For callers that must not allocate device memory themselves or through us:
// host runtimes that hand out all HBM from their own pool and forbid raw
// cudaMalloc (an R or Python serving process that pre-reserves memory for a
// batch of phenotype fits), and latency-critical loops that cannot take the
// device-wide synchronisation cudaMalloc / cudaFree may cause.  Its only
// scratch -- the TF32 high/low halves of the caller's vectors and the tile
// table -- lives in the file-scope array below, sized for at most
// kNoAllocMaxElems vector entries (ncols * np).  Every GPU that loads this
// library holds the array until the process exits.
constexpr int64_t kNoAllocMaxElems = int64_t(1) << 21;  // 2,097,152 entries (e.g. 20 columns at N = 100k)
constexpr int64_t kNoAllocMaxTiles = kNoAllocMaxElems / (kTileM * 32);
constexpr size_t kNoAllocScratchBytes =
    2 * (size_t)kNoAllocMaxElems * sizeof(float) + (size_t)kNoAllocMaxTiles * sizeof(TileCoord);
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

__global__ void noalloc_prepare_kernel(const float* __restrict__ P, int64_t elems, float* __restrict__ hi,
                                       float* __restrict__ lo, TileCoord* __restrict__ tiles,
                                       int64_t nbm, int64_t nbn) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < elems) {
    const float v = P[i];
    const uint32_t u = __float_as_uint(v);
    const float h = isfinite(v) ? __uint_as_float((u + 0x1000u) & 0xFFFFE000u) : v;
    hi[i] = h;
    lo[i] = isfinite(v) ? v - h : 0.0f;
  }
  if (i < nbm * nbn) tiles[i] = TileCoord{(int32_t)(i / nbn), (int32_t)(i % nbn)};
}

// Device address of the scratch array, looked up once per device with that device current.
static cudaError_t noalloc_scratch_ptr(unsigned char** out) {
  constexpr int kMaxDevices = 64;
  static unsigned char* ptrs[kMaxDevices] = {};
  static std::mutex mu;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(mu);
  if (!ptrs[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    ptrs[dev] = static_cast<unsigned char*>(p);
  }
  *out = ptrs[dev];
  return cudaSuccess;
}

int64_t tc_noalloc_max_elems() { return kNoAllocMaxElems; }

cudaError_t tc_gemm_tf32x3_noalloc(const float* Khi, const float* Klo, int64_t np, const float* P,
                                   int64_t ncols, float* Y, cudaStream_t s) {
  if (np % kTileM != 0 || ncols % 32 != 0 || ncols <= 0 || ncols * np > kNoAllocMaxElems)
    return cudaErrorInvalidValue;
  unsigned char* base = nullptr;
  cudaError_t e = noalloc_scratch_ptr(&base);
  if (e != cudaSuccess) return e;
  float* hi = reinterpret_cast<float*>(base);
  float* lo = hi + kNoAllocMaxElems;
  TileCoord* tiles = reinterpret_cast<TileCoord*>(lo + kNoAllocMaxElems);
  const int BN = ncols % 64 == 0 ? 64 : 32;
  const int64_t nbm = np / kTileM, nbn = ncols / BN;
  const int64_t elems = ncols * np;
  const int64_t work = elems > nbm * nbn ? elems : nbm * nbn;
  noalloc_prepare_kernel<<<(unsigned)((work + 255) / 256), 256, 0, s>>>(P, elems, hi, lo, tiles, nbm, nbn);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  CUtensorMap a, b, a2, b2;
  if (!make_map(&a, Khi, true, np, np, (uint64_t)np * 4, kTileM) ||
      !make_map(&a2, Klo, true, np, np, (uint64_t)np * 4, kTileM) ||
      !make_map(&b, hi, true, np, ncols, (uint64_t)np * 4, BN) ||
      !make_map(&b2, lo, true, np, ncols, (uint64_t)np * 4, BN))
    return cudaErrorInvalidValue;
  const int num_kb = (int)(np / 32);
  if (BN == 64)
    e = launch<true, 64, 4, kSplit3>(a, b, a2, b2, tiles, (int)(nbm * nbn), num_kb, drain_stages(128), Y, np, 1.0f,
                                  1, s, np);
  else
    e = launch<true, 32, 5, kSplit3>(a, b, a2, b2, tiles, (int)(nbm * nbn), num_kb, drain_stages(128), Y, np, 1.0f,
                                  1, s, np);
  if (e != cudaSuccess) return e;
  return check_error_flag(s);
}

}  // namespace sg
