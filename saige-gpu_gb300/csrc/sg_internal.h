// Internal declarations shared by the CUDA translation units of libsaigegpu.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>

namespace sg {

// ---- layout helpers
inline int64_t round_up(int64_t x, int64_t a) { return (x + a - 1) / a * a; }
constexpr int kRowTile = 128;   // GRM rows/cols are padded to a multiple of this
constexpr int kMarkerTile = 64; // standardised-genotype columns padded to this (128 B of BF16)
constexpr int kPitchAlign = 16; // byte pitch of packed genotype rows

// ---- counter hash shared with saigegpu/synth.py and the oracle (splitmix64 finaliser x3)
__host__ __device__ inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__host__ __device__ inline uint64_t hash3(uint64_t seed, uint64_t stream, uint64_t idx) {
  uint64_t h = mix64(seed ^ 0x5851F42D4C957F2Dull);
  h = mix64(h ^ (stream * 0x9E3779B97F4A7C15ull));
  return mix64(h ^ (idx * 0xD1B54A32D192ED03ull));
}

// ---- genotype kernels (k_geno.cu)
struct MarkerQC {
  int32_t allele;   // allele count after the integer fill
  int32_t mac;
  int32_t nmiss;
  float freq;       // altFreq over Nnomissing (second estimate)
  float invstd;
  int32_t fill;     // int(round(2p)) replacement for missing calls
  int32_t pass_qc;  // GRM marker
  int32_t pass_vr;  // variance-ratio marker
};

// max_mac_vr != -1 selects categorical variance-ratio markers (every marker with min <= MAC < max)
void launch_marker_qc(const uint8_t* raw, int64_t raw_pitch, int64_t m, int64_t n_fam,
                      const uint32_t* maskbits, int64_t nn, float min_maf, float max_miss,
                      const uint8_t* vr_flag, float min_mac_vr, float max_mac_vr, int is_var_ratio,
                      MarkerQC* out, cudaStream_t s);
// qc == nullptr keeps missing calls (code 01) instead of writing the fill genotype's code
void launch_repack(const uint8_t* raw, int64_t raw_pitch, const int32_t* src_marker,
                   const MarkerQC* qc, int64_t m_out, const int32_t* sub0, int64_t nn,
                   int identity, uint8_t* out, int64_t out_pitch, cudaStream_t s);
void launch_lut(const MarkerQC* qc, const int32_t* src_marker, int64_t m_out, float* lut4,
                cudaStream_t s);
// Z (np x mp, row = sample, markers contiguous) from packed genotypes
void launch_zbuild_f32(const uint8_t* packed, int64_t pitch, const float* lut4, int64_t m_qc,
                       int64_t nn, int64_t np, int64_t mp, float* Z, cudaStream_t s);
void launch_zbuild_bf16(const uint8_t* packed, int64_t pitch, const float* lut4, int64_t m_qc,
                        int64_t nn, int64_t np, int64_t mp, void* Zhi, void* Zlo, cudaStream_t s);
// FP32 diagonal in the reference's marker order and a fixed-point (2^-frac_bits) one beside it;
// scratch holds 12 * 4 * m_qc bytes (16-byte aligned).
void launch_diag(const uint8_t* packed, int64_t pitch, const float* lut4, int64_t m_qc,
                 int64_t nn, int frac_bits, void* scratch, double* diag64, float* diag32,
                 cudaStream_t s);
void launch_synth_bed(uint64_t seed, int64_t n, int64_t m, uint32_t miss_thr16, uint8_t* out,
                      cudaStream_t s);
void launch_genetic_value(const uint8_t* packed, int64_t pitch, const float* lut4, int64_t m_qc,
                          int64_t nn, uint64_t seed, double* out, cudaStream_t s);
void launch_zbuild_marker_major(const uint8_t* packed, int64_t pitch, const float* lut4, int64_t m,
                                int64_t m_rows, int64_t nn, int64_t np, float* Zm, cudaStream_t s);
void launch_loco_combine(float* Yf, double* Yd, const float* V, double a, double b, int64_t n,
                         cudaStream_t s);
void launch_unpack_marker(const uint8_t* packed_row, int64_t nn, const float* lut4, int32_t* g,
                          float* z, cudaStream_t s);

// ---- SIMT GEMM (k_gemm_simt.cu): C = scale * A B^T, A (M x K) and B (N x K) row-major.
// mode 0: C (M x N) row-major; mode 1: C^T stored (N x M, ldc along M);
// mode 2: symmetric rank-k update, A == B, only tiles with block j <= block i computed and
// mirrored.  Requires K % 8 == 0, lda/ldb % 4 == 0, M % 128 == 0, N % BN == 0.
void launch_gemm_nt_f32(const float* A, int64_t lda, const float* B, int64_t ldb, float* C,
                        int64_t ldc, int64_t M, int64_t N, int64_t K, float scale, int mode,
                        cudaStream_t s);
void launch_gemv_f64(const float* K, int64_t ld, int64_t n, const double* x, double* y,
                     cudaStream_t s);

// ---- tcgen05 GEMM (k_tc.cu); returns false when the shape is unsupported.
bool tc_available();
// K = scale * Z Z^T over lower-triangle tiles, Z bf16 (np x mp), K fp32 (np x np).  With
// Zlo != nullptr (Z = Zhi + Zlo split) it accumulates Zhi Zhi^T + Zhi Zlo^T + Zlo Zhi^T.
cudaError_t tc_syrk_bf16(const void* Zhi, const void* Zlo, int64_t np, int64_t mp, float* K,
                         float scale, cudaStream_t s);
// Y^T (ncols x np) = K (np x np fp32, tf32 MMA) * P^T with P (ncols x np fp32).  With Klo and
// Plo (split operands) it accumulates K P + K Plo + Klo P (3xTF32).  With check = false it only
// launches (no stream synchronisation); the caller then reads the kernels' wait-error flag with
// tc_check_error after the stream has drained.
cudaError_t tc_gemm_tf32(const float* K, const float* Klo, int64_t np, const float* P,
                         const float* Plo, int64_t ncols, float* Y, cudaStream_t s, bool check = true);
// Y^T = (Kh + Kl)(Ph + Pl)^T without the Kl Pl term, all four BF16 (kind::f16): 16-bit operand
// significands at the BF16 tensor rate, K in 4 bytes per entry.
// With colmap, tile column j is written to column colmap[j] of Y (skipped when negative).
cudaError_t tc_gemm_bf16x3(const void* Kh, const void* Kl, int64_t np, const void* Ph, const void* Pl,
                           int64_t ncols, float* Y, cudaStream_t s, bool check = true,
                           const int32_t* colmap = nullptr);
// (hi, lo) column j = BF16 halves of column cols[j] of x (np rows, np % 128 == 0), zeros if cols[j] < 0
void launch_split_bf16_gather(const float* x, int64_t np, const int32_t* cols, int64_t ncols, void* hi,
                              void* lo, cudaStream_t s);
// x (+ x2 when not null) = hi + lo, both BF16 (round to nearest even), lo = bf16(x - hi)
void launch_split_bf16(const float* x, const float* x2, void* hi, void* lo, int64_t n, cudaStream_t s);
// Synchronises s, then reads and clears the flag the tcgen05 kernels set when a bounded wait ran
// out (cudaErrorLaunchTimeout in that case).
cudaError_t tc_check_error(cudaStream_t s);
// Runs the kernels' bounded mbarrier wait on a barrier nothing arrives at (budget in ms).
cudaError_t tc_wait_selftest(double budget_ms, int* waited_out, cudaStream_t s);
// Shape options of the tcgen05 GEMMs (process-wide), in the order of sg_tc_option (saigegpu.h):
// SYRK on CTA pairs, split-BF16 GRM.V on CTA pairs, drain length (bytes of K per row per TMEM
// accumulator chunk), SYRK raster group (row tiles), split-BF16 GRM.V K slice bytes (0 = by width).
// Then the subset-exact genotype GEMMs on CTA pairs (0 never, 1 always, 2 above 160 columns) and
// their K slice bytes (0 = by width).
enum { kTcSyrkPair = 0, kTcGrmvPair = 1, kTcDrainBytes = 2, kTcSyrkGroup = 3, kTcGrmvSlice = 4, kTcSubsetPair = 5,
       kTcSubsetSlice = 6, kTcOptions = 7 };
bool tc_set_option(int opt, int value);
int tc_get_option(int opt);
// Split-BF16 GRM.V choices per launch width (n buckets, max_cols increasing; n = 0 clears).
bool tc_set_grmv_plan(const int32_t* max_cols, const int32_t* pair, const int32_t* slice, int n);
int tc_get_grmv_plan(int32_t* max_cols, int32_t* pair, int32_t* slice, int cap);
// The same for the subset-exact engine's genotype GEMMs (slice 64, 128, 256 or 512).
bool tc_set_subset_plan(const int32_t* max_cols, const int32_t* pair, const int32_t* slice, int n);
int tc_get_subset_plan(int32_t* max_cols, int32_t* pair, int32_t* slice, int cap);
// GRM.V column-tile width sets: plain TF32 / FP32, split-TF32, split-BF16 (multiples of 16), and
// the subset-exact genotype GEMMs (multiples of 32)
enum { kTilesPlain = 0, kTilesSplitTF32 = 1, kTilesSplitBF16 = 2, kTilesSplitB = 3 };
// D (ncols x ldd, RHS-major) = A (rows x kdim, exact BF16) (Bh + Bl)^T (ncols x kdim BF16 halves).
// site (0 or 1): which of two call sites queued back to back on one stream (own tile tables).
cudaError_t tc_gemm_splitb(const void* A, int64_t rows, int64_t kdim, const void* Bh, const void* Bl,
                           int64_t ncols, float* D, int64_t ldd, cudaStream_t s, bool check, int site);
// The same with FP16 high halves and E4M3 low halves (A in FP16 and in E4M3, kdim a multiple of 128)
cudaError_t tc_gemm_splitb8(const void* A, const void* A8, int64_t rows, int64_t kdim, const void* Bh,
                            const void* Bl8, int64_t ncols, float* D, int64_t ldd, cudaStream_t s, bool check,
                            int site);
// Column tile width the GRM.V kernel uses for ncols columns.
int tc_gemm_tile_n(int64_t ncols, int set);
// Columns a GRM.V launch covers for ncols live columns (a multiple of 32, or of 16 for split-BF16),
// padded to the width a cost model picks, at most cap.
int64_t tc_grmv_padded_cols(int64_t ncols, int64_t cap, int64_t np, int set, int num_sms);
// Split-TF32 GRM.V that allocates nothing: scratch in a static device array (k_tc.cu).
int64_t tc_noalloc_max_elems();
cudaError_t tc_gemm_tf32x3_noalloc(const float* Khi, const float* Klo, int64_t np, const float* P,
                                   int64_t ncols, float* Y, cudaStream_t s);
// x = hi + lo with hi rounded to TF32 (low 13 mantissa bits zero) and lo = x - hi (exact)
void launch_split_tf32(const float* x, float* hi, float* lo, int64_t n, cudaStream_t s);

// ---- PCG engine kernels (k_pcg.cu)
struct ColState {
  int32_t pheno;    // phenotype slot
  int32_t kind;     // 0 = PCG, 1 = product only, -1 = free
  int32_t active;   // 1 while iterating
  int32_t iter;
  int32_t maxiter;
  int32_t just_done;
  double tol;
  double rz;        // r'z of the current iterate
  double r2;        // r'r
  double alpha, beta;
};
struct PhenoState {
  double tau0, tau1;
};
void launch_pcg_init(int64_t np, int64_t ncols, const int32_t* cols, int64_t ncols_sel,
                     ColState* st, const PhenoState* ph, const double* minv, const double* B,
                     double* X, double* R, double* Z, double* P, float* Pf, double* part,
                     int64_t nblk, cudaStream_t s);
// The step kernels act on ncols columns: cols[0..ncols) when cols is not null (the active list),
// else columns 0..ncols-1.
void launch_pcg_sigma_dot(int64_t np, int64_t ncols, ColState* st, const PhenoState* ph,
                          const double* winv, const double* minv, const double* P,
                          const float* Yf, const double* Yd, double* part, int64_t nblk,
                          const int32_t* cols, cudaStream_t s);
void launch_pcg_alpha(int64_t ncols, ColState* st, const double* part, int64_t nblk,
                      const int32_t* cols, cudaStream_t s);
void launch_pcg_update(int64_t np, int64_t ncols, ColState* st, const PhenoState* ph,
                       const double* winv, const double* minv, double* X, double* R, double* Z,
                       const double* P, const float* Yf, const double* Yd, double* part,
                       int64_t nblk, const int32_t* cols, cudaStream_t s);
void launch_pcg_beta(int64_t ncols, ColState* st, const double* part, int64_t nblk,
                     const int32_t* cols, cudaStream_t s);
void launch_pcg_dir(int64_t np, int64_t ncols, ColState* st, const double* Z, double* P,
                    float* Pf, const int32_t* cols, cudaStream_t s);
void launch_probe_fill(int64_t np, int64_t nn, uint64_t seed, int64_t run0, int64_t k,
                       double* B, cudaStream_t s);
void launch_probe_fill_multi(int64_t np, int64_t nn, const uint64_t* seeds, const int64_t* runs,
                             const int32_t* sel, int64_t k, double* B, cudaStream_t s);
void launch_f64_to_f32(const double* a, float* b, int64_t n, cudaStream_t s);
// d_st[cols[k]] = src[k] for k < n; with Pf, columns set free (kind -1) also get P = 0
void launch_scatter_states(const ColState* src, const int32_t* cols, int64_t n, ColState* dst, float* Pf,
                           int64_t np, cudaStream_t s);
// B[:, sel[k]] = the nn doubles at mapped pinned host address src[k], zero-padded to np
void launch_gather_rhs(const double* const* src, const int32_t* sel, int64_t n, int64_t nn, int64_t np, double* B,
                       cudaStream_t s);
// 1/W and 1/diag(Sigma) of a phenotype slot from W on the device (mask: nullptr = every sample)
void launch_slot_weights(int64_t np, int64_t nn, const double* w, const uint8_t* mask, const double* diag,
                         double m, double tau0, double tau1, int diag_one, double* winv, double* minv,
                         cudaStream_t s);
void launch_f32_to_f64(const float* a, double* b, int64_t n, cudaStream_t s);
int64_t pcg_nblk(int64_t np);

// ---- subset-exact GRM.V (k_subset.cu): per-slot state of a phenotype's sample subset
struct SubsetSlot {
  const float* dprime;    // mg: 1/sd'^2 of the subset's GRM markers, 0 for the others
  const float* p2;        // mg: 2 p' (the subset's allele frequency, FP32 as the reference's LUT)
  const int32_t* flips;   // nflip markers whose subset fill differs from the cohort fill in G
  const float* dfill;     // nflip: subset fill - cohort fill
  const uint32_t* bits;   // W x np (word-major): bit b of word w of sample i = i misses marker
                          // flips[32 w + b] (i in S)
  int32_t nflip = 0, W = 0;
  double inv_m = 0.0;     // 1 / M' (the subset's GRM marker count)
  double ns = 1.0;        // subset size
};
// form 0: BF16 G (Gmm16, Gsm16); form 1: FP16 G (Gmm16, Gsm16) and E4M3 G (Gmm8, Gsm8)
void launch_gbuild(const uint8_t* codes, int64_t pitch, const int32_t* fill, int64_t m, int64_t nn, int64_t mg,
                   int64_t np, int form, void* Gmm16, void* Gsm16, void* Gmm8, void* Gsm8, cudaStream_t s);
// the subset's d', 2p', diagonal table, fill-change list and counts (nflip, M') from its QC records;
// flag: mg bytes of scratch, flips / dfill: room for m entries, counts: 2 int64 on the device;
// markers ex_lo..ex_hi are left out of the subset's GRM (none when ex_lo > ex_hi)
void launch_subset_derive(const MarkerQC* qc, const int32_t* fill_all, int64_t m, int64_t mg, int64_t ex_lo,
                          int64_t ex_hi, float* dp, float* p2, float* lut4, uint8_t* flag, int32_t* flips, float* dfill,
                          int64_t* counts, cudaStream_t s);
void launch_subset_bitmap(const uint8_t* codes, int64_t pitch, const int32_t* flips, int nflip, int W,
                          const uint8_t* mask, int64_t nn, int64_t np, uint32_t* bits, cudaStream_t s);
// part: subset_diag_scratch(m, np) floats of scratch
int64_t subset_diag_scratch(int64_t m, int64_t np);
void launch_subset_diag(const uint8_t* codes, int64_t pitch, const float* lut4, int64_t m, int64_t nn, int64_t np,
                        float* part, double* out, cudaStream_t s);
int subset_nblk(int64_t n);
// per step: column sums over the subset, then the centred BF16 halves (compact block of ncols)
void launch_subset_prepare(const float* Pf, int64_t np, const int32_t* cols, int64_t ncols, const ColState* st,
                           const SubsetSlot* slots, const double* winv, double* part, void* Vh, void* Vl,
                           cudaStream_t s);
// after GEMM 1: fill corrections into T, then T' = d' .* T as halves and the (2p')^T T' partials
void launch_subset_scale(const void* Vh, const void* Vl, int64_t np, int64_t nn, const int32_t* cols, int64_t ncols,
                         const ColState* st, const SubsetSlot* slots, int max_w, float* T, int64_t mg, void* Th,
                         void* Tl, double* part, cudaStream_t s);
// after GEMM 2: Y[cols[j]] = (U + dF T' - (2p')^T T') / M' on the subset
void launch_subset_finalize(const float* U, int64_t np, int64_t nn, const int32_t* cols, int64_t ncols,
                            const ColState* st, const SubsetSlot* slots, const void* Th, const void* Tl, int64_t mg,
                            const double* part, const double* winv, float* Yf, cudaStream_t s);
// FP16-high / E4M3-low form of the same three steps; pmax: block maxima scratch (as part), scale:
// 2 x cap floats (s1 of compact column j at j, s2 at cap + j)
void launch_subset_prepare_f8(const float* Pf, int64_t np, const int32_t* cols, int64_t ncols, const ColState* st,
                              const SubsetSlot* slots, const double* winv, double* part, float* pmax, void* Vh,
                              void* Vl, float* scale, cudaStream_t s);
void launch_subset_scale_f8(const void* Vh, const void* Vl, int64_t np, int64_t nn, const int32_t* cols,
                            int64_t ncols, const ColState* st, const SubsetSlot* slots, int max_w, float* T,
                            int64_t mg, void* Th, void* Tl, double* part, float* pmax, float* scale, int64_t cap,
                            cudaStream_t s);
void launch_subset_finalize_f8(const float* U, int64_t np, int64_t nn, const int32_t* cols, int64_t ncols,
                               const ColState* st, const SubsetSlot* slots, const void* Th, const void* Tl,
                               int64_t mg, const float* scale2, const double* part, const double* winv, float* Yf,
                               cudaStream_t s);
constexpr int kProbeDotsMaxP = 16;
// Per probe j (vecs[j] = Sigma^-1 u_j and vecs[k+j] = K u_j, u masked by minv != 0):
// block partials of [Au.Su, u.Su, Au.SX_q (q < p), SX_q.u (q < p)] -> part[(j*nblk + b)*(2+2p) + v]
void launch_probe_dots(int64_t np, int64_t nn, const double* const* vecs, int64_t k,
                       const double* minv_row, uint64_t seed, int64_t run0, const double* SX,
                       int64_t p, double* part, int64_t nblk, cudaStream_t s);

}  // namespace sg
