/*
 * saigegpu.h -- C ABI of the GB300-native SAIGE step-1 hot path.
 *
 * One context owns one GPU, the decoded genotypes, the dense GRM resident in
 * HBM and a multi-RHS PCG engine.  Every entry point returns an int status
 * (SG_OK == 0); no C++ exception crosses the ABI.  Host buffers are owned by
 * the caller; device memory is owned by the context.  A context is not
 * thread-safe: use one per host thread, or serialise calls.
 *
 * Each entry point names the reference interface it replaces (paths relative
 * to the reference project; "FIT.cpp" = src/SAIGE/src/SAIGE_fitGLMM_fast.cpp,
 * "RcppExports.cpp" = src/SAIGE/src/RcppExports.cpp).  The reference passes
 * Armadillo float vectors; the *_f32 drop-ins keep that, and FP64 variants
 * exist for the mixed-precision path.
 *
 * Vector layout: a block of k vectors of length n is "RHS-major": vector j
 * occupies [j*n, (j+1)*n).  Matrices X (n x p) follow the same convention
 * (column j contiguous), which is Armadillo's column-major layout.
 */
#ifndef SAIGEGPU_H
#define SAIGEGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sg_ctx sg_ctx;

enum sg_status {
  SG_OK = 0,
  SG_ERR_INVALID = 1,   /* bad argument or size */
  SG_ERR_CUDA = 2,      /* CUDA runtime / launch failure */
  SG_ERR_NOMEM = 3,     /* device allocation refused (incl. the context's HBM budget) */
  SG_ERR_STATE = 4,     /* call out of order (e.g. no genotypes / no GRM yet) */
  SG_ERR_IO = 5,        /* file could not be read */
  SG_ERR_NUMERIC = 6,   /* NaN/Inf in inputs or a singular system */
  SG_ERR_NOT_FOUND = 7, /* unknown request id */
  SG_ERR_TIMEOUT = 8    /* a bounded device wait gave up */
};

/* GRM build precisions (sg_grm_build) */
enum sg_grm_precision {
  SG_GRM_FP32_SIMT = 0, /* FP32 standardised genotypes, FP32 CUDA-core SYRK */
  SG_GRM_BF16_TC = 1,   /* BF16 genotypes, tcgen05 SYRK, FP32 accumulation in TMEM */
  SG_GRM_BF16X3_TC = 2  /* split-BF16 (hi+lo, 4 products) tcgen05 SYRK: 16-bit genotypes, near-FP64 K */
};

/* GRM.V product engines used inside the PCG (sg_set_matvec_mode) */
enum sg_matvec_mode {
  SG_MV_FP32_SIMT = 0,  /* FP32 K, FP32 operands, CUDA cores */
  SG_MV_TF32_TC = 1,    /* tcgen05 kind::tf32 on the FP32 K: one product, ~2^-11 relative per term */
  SG_MV_FP64_PLAIN = 2, /* plain FP64 GEMV (the single-RHS baseline) */
  SG_MV_TF32X3_TC = 3,  /* split-TF32 on tcgen05: K = Khi + Klo, P = Phi + Plo, three products
                           accumulated in TMEM (FP32-class accuracy at tensor-core rate) */
  SG_MV_BF16X3_TC = 4,  /* split-BF16 on tcgen05 (kind::f16): K and P as BF16 high + low halves
                           (16 significant bits), three products in TMEM; ~1.5e-5 relative per
                           term, half the bytes and twice the MMA rate of SG_MV_TF32X3_TC */
  SG_MV_SUBSET_EXACT = 5 /* subset-exact: each phenotype slot's product is K_S P with K_S the GRM
                            of the slot's own sample subset (its allele frequencies, fill, QC and
                            1/sd, as setgeno over that subset computes them, FIT.cpp:376-385,
                            436-495), applied through the genotype matrix (0/1/2 in BF16, exact)
                            with two tcgen05 GEMMs of two BF16 products each; needs no sg_grm_build.
                            The other engines restrict the cohort GRM to the subset instead */,
  SG_MV_SUBSET_EXACT_F8 = 6 /* the subset-exact engine with FP16 high halves (kind::f16) and E4M3
                            low halves (kind::f8f6f4, twice the FP16 rate) of each column scaled
                            by a power of two: 15 significant bits, three quarters of the tensor
                            work; G is held in FP16 and in E4M3 (1.5 times the bytes).  Measured
                            at N = 100k: 3-5% faster GRM.V than SG_MV_SUBSET_EXACT, K_S v within
                            1.1e-5 of FP64 (5e-6 for the BF16 form), tau up to 1.6e-4 from FP64 on
                            a test cohort (1e-6 for the BF16 form); not the default */
};

/* ------------------------------------------------------------ context */
int sg_ctx_create(int device, uint64_t hbm_budget_bytes, sg_ctx **out);
void sg_ctx_destroy(sg_ctx *ctx);
/* Make the context's GPU current on the calling host thread; a caller that drives one context
 * from several threads (calls serialised by the caller) does this once per thread.  No reference
 * counterpart (the reference is single-threaded at this boundary). */
int sg_ctx_make_current(sg_ctx *ctx);
const char *sg_last_error(const sg_ctx *ctx);
int sg_device_bytes_in_use(const sg_ctx *ctx, uint64_t *bytes);
int sg_set_matvec_mode(sg_ctx *ctx, int mode);
/* Failure-detection self-test: runs the tcgen05 kernels' bounded mbarrier wait on a barrier that
 * nothing arrives at, with a budget of budget_ms (<= 2000).  Returns SG_ERR_TIMEOUT (the expected
 * outcome) through the same device error flag the GEMMs use; the context stays usable. */
int sg_selftest_wait_timeout(sg_ctx *ctx, double budget_ms);
/* Shape options of the tcgen05 GEMMs (process-wide; saigegpu.tune picks them by timing).  No
 * reference counterpart (the reference's GRM.x is two cuBLAS SGEMV calls, gpuSymMatMult.cu:211-252).
 * Every choice gives the same products up to the drain length: the accumulation order within a
 * drain chunk and across chunks does not depend on the others. */
enum sg_tc_option {
  SG_TC_SYRK_PAIR = 0,   /* 1: SYRK tiles of 256 x 256 on CTA pairs (tcgen05 cta_group::2), the
                            default (1.31 s against 1.38 s on single CTAs at N = 100k, M = 150k) */
  SG_TC_GRMV_PAIR = 1,   /* 1: split-BF16 GRM.V tiles of 256 rows on CTA pairs; default 0 */
  SG_TC_DRAIN_BYTES = 2, /* bytes of K per row one TMEM accumulator takes before it is added into
                            registers: 128..4096, a multiple of 128; default 512 */
  SG_TC_SYRK_GROUP = 3,  /* row tiles per raster group of the SYRK (1..4096); default 8 */
  SG_TC_GRMV_SLICE = 4,  /* K slice bytes per pipeline stage of the split-BF16 GRM.V: 0 = by
                            width (128 up to 160 columns, else 64), 64 or 128; default 0 */
  SG_TC_SUBSET_PAIR = 5, /* the subset-exact engine's genotype GEMMs on CTA pairs: 0 never,
                            1 always, 2 above 160 columns (default) */
  SG_TC_SUBSET_SLICE = 6 /* their K slice bytes per pipeline stage: 0 = by width (128 up to 160
                            columns, else 64), 64, 128, 256 (default: two 128-byte boxes per
                            operand and stage) or 512 (four); a width without room for two such
                            stages runs the next smaller one (256 above 160 columns on single
                            CTAs: 128; 512 beyond 32-column tiles, or 64 on pairs: 256) */
};
int sg_set_tc_option(sg_ctx *ctx, int option, int value);
int sg_get_tc_option(sg_ctx *ctx, int option, int *value);
/* Per-width plan of the split-BF16 GRM.V (the tuner's choice table; process-wide): a launch over
 * ncols columns takes pair[i] (SG_TC_GRMV_PAIR) and slice[i] (SG_TC_GRMV_SLICE) of the first
 * bucket i with ncols <= max_cols[i] (max_cols increasing; at most 64 buckets); wider launches use
 * the options.  n = 0 clears the plan.  sg_get_grmv_plan copies up to cap buckets and sets *n to
 * the plan's length.  No reference counterpart. */
int sg_set_grmv_plan(sg_ctx *ctx, int n, const int32_t *max_cols, const int32_t *pair,
                     const int32_t *slice);
int sg_get_grmv_plan(sg_ctx *ctx, int cap, int32_t *max_cols, int32_t *pair, int32_t *slice, int *n);
/* The same per-width table for the subset-exact engine's genotype GEMMs (SG_TC_SUBSET_PAIR and
 * SG_TC_SUBSET_SLICE per bucket; slice 64, 128, 256 or 512).  No reference counterpart. */
int sg_set_subset_plan(sg_ctx *ctx, int n, const int32_t *max_cols, const int32_t *pair,
                       const int32_t *slice);
int sg_get_subset_plan(sg_ctx *ctx, int cap, int32_t *max_cols, int32_t *pair, int32_t *slice, int *n);
/* GPU kernel launches issued by this context so far (for accounting). */
int sg_kernel_launches(const sg_ctx *ctx, uint64_t *count);

/* ------------------------------------------------------------ genotypes
 * Replaces setgeno (FIT.cpp:2267-2275 -> genoClass::setGenoObj FIT.cpp:739-1024;
 * RcppExports.cpp:725-737).  ``bed`` is the whole .bed file (with its 3-byte
 * magic).  ``sub_1based``: subSampleInGeno (1-based .fam positions, analysis
 * order).  ``pheno_mask``: indicatorGenoSamplesWithPheno (n_fam bytes).
 * ``vr_random_markers``: the marker indices (0-based) of the random draw that
 * the reference makes with arma::randi (FIT.cpp:866-868); markers in it with
 * MAC >= min_mac_vr leave the GRM when is_var_ratio != 0 (FIT.cpp:521-547).
 * Thresholds mirror setminMAFforGRM / setmaxMissingRateforGRM
 * (FIT.cpp:4923-4930) and setminMAC_VarianceRatio (FIT.cpp:4970).
 */
int sg_setgeno(sg_ctx *ctx, const uint8_t *bed, uint64_t bed_len, int64_t n_fam, int64_t m_bim,
               const int32_t *sub_1based, int64_t n_sub, const uint8_t *pheno_mask,
               float min_maf, float max_missing, const int32_t *vr_random_markers,
               int64_t n_vr_random, float min_mac_vr, int is_var_ratio, int is_diag_one);
/* Categorical variance ratios for the next setgeno: the upper MAC bound g_maxMACVarRatio of
 * setminMAC_VarianceRatio (FIT.cpp:4969-4973; the lower bound is setgeno's min_mac_vr).  With
 * max_mac != -1, every marker with min_mac_vr <= MAC < max_mac becomes a variance-ratio marker and
 * leaves the GRM, and from max_mac up only the random draw's markers do (FIT.cpp:497-518).
 * -1 (the default) keeps the single-ratio selection. */
int sg_set_vr_max_mac(sg_ctx *ctx, float max_mac);
/* Same, reading the files; n_fam / m_bim are the line counts of .fam / .bim (FIT.cpp:760-787). */
int sg_setgeno_files(sg_ctx *ctx, const char *bed_path, const char *bim_path, const char *fam_path,
                     const int32_t *sub_1based, int64_t n_sub, const uint8_t *pheno_mask,
                     float min_maf, float max_missing, const int32_t *vr_random_markers,
                     int64_t n_vr_random, float min_mac_vr, int is_var_ratio, int is_diag_one);
/* Uses a .bed image already in device memory (e.g. from sg_synth_bed). */
int sg_setgeno_device(sg_ctx *ctx, const uint8_t *bed_dev, uint64_t bed_len, int64_t n_fam,
                      int64_t m_bim, const int32_t *sub_1based, int64_t n_sub,
                      const uint8_t *pheno_mask, float min_maf, float max_missing,
                      const int32_t *vr_random_markers, int64_t n_vr_random, float min_mac_vr,
                      int is_var_ratio, int is_diag_one);
/* n = Nnomissing, m_total = M of the .bim, m_qc = GRM markers, m_vr = variance-ratio markers */
int sg_geno_dims(sg_ctx *ctx, int64_t *n, int64_t *m_total, int64_t *m_qc, int64_t *m_vr);
/* getAlleleFreqVec / invstdvVec / getMACVec (RcppExports.R:128-160): length m_qc */
int sg_get_allele_freq(sg_ctx *ctx, float *out);
int sg_get_invstd(sg_ctx *ctx, float *out);
int sg_get_mac(sg_ctx *ctx, int32_t *out);
/* getQCdMarkerIndex: m_total bytes, 1 for GRM markers */
int sg_get_qc_marker_mask(sg_ctx *ctx, uint8_t *out);
/* variance-ratio markers: freq, MAC and .bim index (getMACVec_forVarRatio, getIndexVec_forVarRatio) */
int sg_get_vr_markers(sg_ctx *ctx, float *freq, int32_t *mac, int32_t *bim_index);
/* re-packed 2-bit GRM genotypes, m_qc rows of ceil(n/4) bytes (genoVecofPointers) */
int sg_get_packed_geno(sg_ctx *ctx, uint8_t *out);
/* Get_OneSNP_Geno (FIT.cpp:223-273) / Get_OneSNP_Geno_forVarRatio (FIT.cpp:275-323) / Get_OneSNP_StdGeno (FIT.cpp:582-662) */
int sg_get_onesnp_geno(sg_ctx *ctx, int64_t marker, int32_t *out);
int sg_get_onesnp_geno_vr(sg_ctx *ctx, int64_t marker, int32_t *out);
int sg_get_onesnp_stdgeno(sg_ctx *ctx, int64_t marker, float *out);

/* ------------------------------------------------------------ GRM
 * Builds K = Z Z' / M_qc in HBM (the reference never forms K; it applies
 * Z_r(Z_r' x) per call, FIT.cpp:1635-1708 and gpuSymMatMult.cu:211-252).
 */
int sg_grm_build(sg_ctx *ctx, int precision);
/* Device time (CUDA events) of the last setgeno / grm_build, ms: [0] per-marker QC, [1] re-pack +
 * LUT, [2] GRM diagonal, [3] standardised-genotype build, [4] SYRK. */
int sg_build_timing(sg_ctx *ctx, double *t5);
/* Get_Diagof_StdGeno (FIT.cpp:665-704): sum_m z^2 per sample.  The f32 form is
 * accumulated in marker order in float exactly as the reference does. */
int sg_grm_diag(sg_ctx *ctx, double *out);
int sg_grm_diag_f32(sg_ctx *ctx, float *out);
/* Copy the n x n GRM to the host (row-major; small n only). */
int sg_grm_get(sg_ctx *ctx, float *out);
/* K V for k vectors (RHS-major, FP64 in and out; the product runs in FP32). */
int sg_grm_matmul(sg_ctx *ctx, const double *V, int64_t k, double *out);

/* GRM.V for callers that cannot allocate device memory.  No counterpart in the reference: it exists
 * for host runtimes that own all device memory through their own pool and forbid cudaMalloc, and
 * for latency-critical loops that cannot absorb the synchronisation cudaMalloc/cudaFree can cause.
 * Y (ncols x n_p, RHS-major, device) = K P with P (ncols x n_p FP32, RHS-major, device); n_p = n
 * rounded up to 128 (sg_grm_padded_n), rows past n of P must be zero.  Runs the split-TF32 tcgen05
 * product, so the context must already be in SG_MV_TF32X3_TC mode (else SG_ERR_STATE: switching
 * would allocate).  The call allocates nothing: its scratch is one static device array of
 * 2 x 2^21 floats plus a tile table (about 16 MiB), so ncols * n_p must not exceed 2,097,152 and
 * ncols must be a multiple of 32 (else SG_ERR_INVALID).  The first call on a device looks up that
 * array's device address, so make the first call before any stream capture.  Every call shares
 * the array and overwrites what it uses; calls that overlap on the GPU (e.g. on two streams) race.
 * A bounded device wait that gives up in any tcgen05 GEMM of the process sets one process-wide
 * flag, which the next call that checks it reads and clears: a call that overlaps another tcgen05
 * product on another stream may report that product's timeout, or leave its own to that product.
 * ``stream`` is a cudaStream_t (NULL = the legacy default stream); the call returns after the
 * product has finished. */
int sg_grm_matmul_tf32x3_noalloc(sg_ctx *ctx, const float *P_dev, int64_t ncols, float *Y_dev,
                                 void *stream);
/* GRM row count padded to the tile size (the leading dimension of device-side vector blocks). */
int sg_grm_padded_n(sg_ctx *ctx, int64_t *np);

/* Leave one chromosome out: GRM markers [begin, end] (0-based, inclusive, in GRM-marker order) leave
 * the GRM for every later product and preconditioner until sg_loco_clear.  Replaces
 * setStartEndIndex (FIT.cpp:3067-3085) + parallelCrossProd_LOCO (FIT.cpp:1790-1851) +
 * getDiagOfSigma_LOCO (FIT.cpp:2370-2392): K_-j P = (M K P - Z_j Z_j' P) / (M - M_j) with the
 * chromosome's standardised genotypes in FP32, and diag minus its sum z^2.  The _LOCO drop-ins of
 * the reference (getCoefficients_LOCO, getPCG1ofSigmaAndVector_LOCO, ...) are the plain drop-ins
 * called while a range is set.  Phenotype slots read the diagonal when set, so (re)set them after.
 * The subset-exact engines reject it (their GRM markers differ by phenotype): use sg_loco_set_bim. */
int sg_loco_set(sg_ctx *ctx, int64_t begin, int64_t end);
/* Leave one chromosome out, given as .bim markers [begin, end] (0-based, inclusive).  The GRM
 * markers inside it are those the reference's updateChrStartEndIndexVec (Util.R:29-65) finds for the
 * chromosome.  On a resident GRM this is sg_loco_set over that range of GRM markers.  In the
 * subset-exact engines every phenotype's GRM markers are the .bim markers passing QC over its own
 * samples (setgeno per phenotype, FIT.cpp:376-385), so the range applies per phenotype: a slot set
 * (sg_engine_set_pheno) after this call leaves its own GRM markers inside [begin, end] out of its
 * GRM, its diagonal and its marker count M', as the reference's setStartEndIndex +
 * parallelCrossProd_LOCO + getDiagOfSigma_LOCO (FIT.cpp:3067-3085, 1790-1851, 2370-2392) do over
 * that phenotype's setgeno.  Set every slot again after the call.  sg_loco_clear ends either form. */
int sg_loco_set_bim(sg_ctx *ctx, int64_t begin, int64_t end);
int sg_loco_clear(sg_ctx *ctx);

/* ------------------------------------------------------------ drop-ins for the Rcpp entry points */
/* getCrossprodMatAndKin (FIT.cpp:1953-1981; RcppExports.cpp:664-671) */
int sg_getCrossprodMatAndKin(sg_ctx *ctx, const float *b, float *out);
/* getDiagOfSigma (FIT.cpp:2322-2365; RcppExports.cpp:774-782); tau[2] */
int sg_getDiagOfSigma(sg_ctx *ctx, const float *w, const float *tau, float *out);
/* getCrossprod (FIT.cpp:2397-2425; RcppExports.cpp:798-807) */
int sg_getCrossprod(sg_ctx *ctx, const float *b, const float *w, const float *tau, float *out);
/* getPCG1ofSigmaAndVector (FIT.cpp:2593-2809; RcppExports.cpp:900-911).  iters may be NULL. */
int sg_getPCG1ofSigmaAndVector(sg_ctx *ctx, const float *w, const float *tau, const float *b,
                               int maxiter, float tol, float *out, int32_t *iters);
/* Multi-RHS FP64 solve: k independent columns, each stopped like the reference. */
int sg_pcg_solve(sg_ctx *ctx, const double *w, const double *tau, const double *B, int64_t k,
                 int maxiter, double tol, double *X, int32_t *iters);
/* getSigma_X (FIT.cpp:3347-3366) and getSigma_G (FIT.cpp:3394-3398) */
int sg_getSigma_X(sg_ctx *ctx, const float *w, const float *tau, const float *X, int64_t p,
                  int maxiter, float tol, float *out);
int sg_getSigma_G(sg_ctx *ctx, const float *w, const float *tau, const float *g, int maxiter,
                  float tol, float *out);
/* getCoefficients (FIT.cpp:3167-3199; RcppExports.cpp:1019-1031).  Outputs:
 * Sigma_iY[n], Sigma_iX[n*p], cov[p*p], alpha[p], eta[n]. */
int sg_getCoefficients(sg_ctx *ctx, const float *Y, const float *X, int64_t p, const float *w,
                       const float *tau, int maxiter, float tol, float *Sigma_iY, float *Sigma_iX,
                       float *cov, float *alpha, float *eta);
/* GetTrace (FIT.cpp:3113-3160; RcppExports.cpp:1000-1015).  Probes: counter hash of
 * (probe_seed, run, sample), the reference's comm.set.seed(200)+rbinom stream stand-in. */
int sg_GetTrace(sg_ctx *ctx, const float *Sigma_iX, const float *X, int64_t p, const float *w,
                const float *tau, const float *cov, int nrun, int maxiter, float tol,
                float trace_cv_cutoff, uint64_t probe_seed, float *trace, int32_t *nrun_used);
/* GetTrace_q (FIT.cpp:3409-3472): trace[0] = tr(P), trace[1] = tr(PK) */
int sg_GetTrace_q(sg_ctx *ctx, const float *Sigma_iX, const float *X, int64_t p, const float *w,
                  const float *tau, const float *cov, int nrun, int maxiter, float tol,
                  float trace_cv_cutoff, uint64_t probe_seed, float *trace, int32_t *nrun_used);
/* getAIScore (FIT.cpp:3279-3295; RcppExports.cpp:1067-1084): YPAPY, Trace, AI and PY[n]. */
int sg_getAIScore(sg_ctx *ctx, const float *Y, const float *X, int64_t p, const float *w,
                  const float *tau, const float *Sigma_iY, const float *Sigma_iX, const float *cov,
                  int nrun, int maxiter, float tol, float trace_cv_cutoff, uint64_t probe_seed,
                  float *YPAPY, float *Trace, float *AI, float *PY);
/* getAIScore_q (FIT.cpp:3479-3531): YPAPY, YPA0PY, Trace[2], AI[4] (col-major 2x2), PY[n] */
int sg_getAIScore_q(sg_ctx *ctx, const float *Y, const float *X, int64_t p, const float *w,
                    const float *tau, const float *Sigma_iY, const float *Sigma_iX,
                    const float *cov, int nrun, int maxiter, float tol, float trace_cv_cutoff,
                    uint64_t probe_seed, float *YPAPY, float *YPA0PY, float *Trace, float *AI,
                    float *PY);
/* fitglmmaiRPCG (FIT.cpp:3302-3341; RcppExports.cpp:1088-1106): tau[2] updated in place */
int sg_fitglmmaiRPCG(sg_ctx *ctx, const float *Y, const float *X, int64_t p, const float *w,
                     float *tau, const float *Sigma_iY, const float *Sigma_iX, const float *cov,
                     int nrun, int maxiter, float tol_pcg, float tol, float trace_cv_cutoff,
                     uint64_t probe_seed);
/* fitglmmaiRPCG_q (FIT.cpp:3610-3662; RcppExports.cpp:1170-1206) */
int sg_fitglmmaiRPCG_q(sg_ctx *ctx, const float *Y, const float *X, int64_t p, const float *w,
                       float *tau, const float *Sigma_iY, const float *Sigma_iX, const float *cov,
                       int nrun, int maxiter, float tol_pcg, float tol, float trace_cv_cutoff,
                       uint64_t probe_seed);

/* ------------------------------------------------------------ batched solve engine
 * Continuous batching of PCG columns over the resident GRM.  A "phenotype
 * slot" holds W, tau and a sample mask; columns (right-hand sides) are
 * admitted against a slot, advance one PCG iteration per engine step together
 * with every other in-flight column, and retire on their own stopping rule
 * (the reference's sum r^2 <= tol or maxiter).  A column's result does not
 * depend on which other columns shared its steps.
 */
int sg_engine_reserve(sg_ctx *ctx, int64_t max_columns, int64_t max_phenos);
/* Define/replace phenotype slot ``slot``: w[n] (0 or NaN-free), tau[2], mask[n] (1 = sample in
 * this phenotype's subset; NULL = all). */
int sg_engine_set_pheno(sg_ctx *ctx, int64_t slot, const double *w, const double *tau,
                        const uint8_t *mask);
/* Subset-exact engine: a slot keeps its subset's state (allele frequencies, fill, QC, 1/sd, the
 * fill-change map and the diagonal; setgeno over the subset, FIT.cpp:376-385, 436-495) while its
 * mask is unchanged, so later sg_engine_set_pheno calls (new weights each AI-REML iteration) only
 * upload weights.  This drops every slot's kept state: the next sg_engine_set_pheno of each slot
 * rebuilds it, as for a new phenotype.  No reference counterpart. */
int sg_engine_forget_subsets(sg_ctx *ctx);
/* Subset-exact engine, for a driver whose threads serialise their engine calls: launch the first,
 * longer half of slot ``slot``'s subset set-up for ``mask`` (QC over the subset, its tables,
 * fill-change list and diagonal) without waiting; sg_engine_subset_wait(slot) then blocks until the
 * counts the host needs are back and, like sg_engine_wait, need not be serialised with other
 * threads' calls; the slot's next sg_engine_set_pheno with the same mask completes the set-up.
 * Both are no-ops when the slot already holds that subset, and sg_engine_prepare_subset is one for
 * the other engines.  Set-ups run on the context's lowest-priority stream, below the engine steps,
 * so they fill SMs the steps leave idle; a driver may prepare a queued phenotype in a spare slot
 * while it waits for room.  No reference counterpart. */
int sg_engine_prepare_subset(sg_ctx *ctx, int64_t slot, const uint8_t *mask);
/* A set-up slot's variance-ratio markers as setgeno over its subset selects them: up to cap .bim
 * indices (marker order) and their MAC over the subset; *n gets the count.  And one .bim marker's
 * genotypes (0/1/2) for every cohort sample with missing calls at the subset's fill
 * (Get_OneSNP_Geno_forVarRatio over the subset).  Subset-exact engines only. */
int sg_engine_subset_vr_markers(sg_ctx *ctx, int64_t slot, int32_t *bim_index, int32_t *mac, int64_t cap,
                                int64_t *n);
int sg_engine_subset_geno(sg_ctx *ctx, int64_t slot, int64_t marker, int32_t *out);
int sg_engine_subset_wait(sg_ctx *ctx, int64_t slot);
/* Queue k columns.  kind 0 = PCG solve of Sigma x = b, kind 1 = one GRM product K b.
 * ids[k] receives request ids. */
int sg_engine_submit(sg_ctx *ctx, int64_t slot, int kind, const double *B, int64_t k, int maxiter,
                     double tol, int64_t *ids);
/* Submit Rademacher probes (counter hash of seed, run0+j, sample) as PCG (kind 0) or product (kind 1) columns. */
int sg_engine_submit_probes(sg_ctx *ctx, int64_t slot, int kind, uint64_t seed, int64_t run0,
                            int64_t k, int maxiter, double tol, int64_t *ids);
/* Queue k PCG solves whose right-hand sides are the results of requests src_ids[k] (e.g. a K b
 * product, solved as Sigma x = K b without a round trip through the host).  Each is admitted at the
 * first launch after its source has finished; if the source is fetched, cancelled or reduced first,
 * its result is copied to the solve's own right-hand side (a source cancelled before it finished
 * cancels the solve).  Needs held results (sg_engine_hold_results).  No reference counterpart. */
int sg_engine_submit_chained(sg_ctx *ctx, int64_t slot, const int64_t *src_ids, int64_t k, int maxiter,
                             double tol, int64_t *ids);
/* Run up to max_steps engine steps (admitting queued columns as slots free up).
 * Returns after the step in which at least one column retired, or when idle. */
int sg_engine_run(sg_ctx *ctx, int64_t max_steps, int64_t *n_finished);
/* Asynchronous stepping (no reference counterpart: the reference's PCG loop, FIT.cpp:2593-2680,
 * blocks on every product).  sg_engine_launch admits queued columns and starts one step without
 * waiting for it (*launched = 0 when nothing is active; *n_finished counts columns that retired
 * at admission); sg_engine_finish waits for that step and retires its finished columns.  Between
 * the two the caller may submit (joins the next launch), poll, fetch or cancel, run
 * sg_engine_probe_dots and upload weights with sg_engine_set_pheno for slots without running
 * columns: those calls use a second stream and do not wait for the step.  sg_engine_run finishes
 * an in-flight step first. */
int sg_engine_launch(sg_ctx *ctx, int64_t *n_finished, int *launched);
int sg_engine_finish(sg_ctx *ctx, int64_t *n_finished);
/* Block until the launched step has run on the device without finishing it.  Unlike every other
 * engine call it need not be serialised with the calls other threads make (the thread that
 * launches and finishes steps calls it); a device error is reported by the next sg_engine_finish. */
int sg_engine_wait(sg_ctx *ctx);
/* By default a finished column's result is copied to the host and its column freed at once.
 * With hold != 0 finished results stay on the device (keeping their column) until fetched,
 * cancelled or consumed by sg_engine_probe_dots; sg_engine_run then fails with SG_ERR_STATE
 * rather than wait forever when queued columns find every column holding a result.  The blocking
 * drop-ins switch holding off. */
int sg_engine_hold_results(sg_ctx *ctx, int hold);
/* Fetch and release a finished column: x[n], iterations.  SG_ERR_STATE if not finished. */
int sg_engine_fetch(sg_ctx *ctx, int64_t id, double *x, int32_t *iters);
int sg_engine_cancel(sg_ctx *ctx, int64_t id);
/* Hutchinson trace reductions on the device for k finished probe pairs (ids_pcg[j] = Sigma^-1 u_j,
 * ids_prod[j] = K u_j, u_j the counter-hash probe of (seed, run0 + j) masked to the slot's samples):
 * out[j*(2+2p) + ...] = [Au.Su, u.Su, Au.SX_0..p-1, SX_0..p-1.u] with SX (n x p, column-major, host)
 * = Sigma^-1 X.  Then tr(PK)_j = Au.Su - b' cov c and tr(P)_j = u.Su - c' cov c (GetTrace /
 * GetTrace_q FIT.cpp:3133-3146, 3427-3446).  Consumes (releases) the 2k results; p <= 16. */
int sg_engine_probe_dots(sg_ctx *ctx, int64_t slot, const int64_t *ids_pcg, const int64_t *ids_prod,
                         int64_t k, uint64_t seed, int64_t run0, const double *SX, int64_t p,
                         double *out, int32_t *iters);
/* The same in three calls, for a driver whose threads serialise their engine calls: _begin checks
 * the requests and launches the reduction without waiting (one per slot at a time); _wait blocks
 * until it has run and, like sg_engine_wait, need not be serialised with other threads' calls;
 * _end writes out and iters and releases the 2k results.  No reference counterpart. */
int sg_engine_probe_dots_begin(sg_ctx *ctx, int64_t slot, const int64_t *ids_pcg, const int64_t *ids_prod,
                               int64_t k, uint64_t seed, int64_t run0, const double *SX, int64_t p);
int sg_engine_probe_dots_wait(sg_ctx *ctx, int64_t slot);
int sg_engine_probe_dots_end(sg_ctx *ctx, int64_t slot, double *out, int32_t *iters);
/* K u of a slot's probes is kept on the device once computed (the probes and the slot's sample mask
 * are fixed during a fit): an ids_prod entry of -1 in sg_engine_probe_dots reads the cached K u of
 * (seed, run0 + j).  Clear a slot's cache when a new phenotype (mask) takes it (slot -1: all). */
int sg_engine_probe_cache_clear(sg_ctx *ctx, int64_t slot);
/* 1 if K u of probe (seed, run) is cached for the slot, else 0. */
int sg_engine_probe_cached(sg_ctx *ctx, int64_t slot, uint64_t seed, int64_t run);
/* Ids of columns that finished since the previous poll (up to max_ids); *n_out gets the count. */
int sg_engine_poll(sg_ctx *ctx, int64_t *ids, int64_t max_ids, int64_t *n_out);
/* counters: [0]=engine steps, [1]=columns retired, [2]=column-iterations, [3]=GRM passes */
int sg_engine_stats(sg_ctx *ctx, int64_t *stats4);
/* device timing from CUDA events on the engine stream:
 * [0]=engine-step device ms, [1]=GRM.V GEMM device ms, [2]=GEMM launches,
 * [3]=algorithmic GEMM FLOPs over the columns processed (2 n^2 each), [4]=columns processed,
 * [5]=occupied (useful) columns processed */
int sg_engine_timing(sg_ctx *ctx, double *t6);
/* ms3[0]: device time between the end of one engine step and the start of the next (CUDA events),
 * summed since the last sg_engine_reset_timing; ms3[1]: the part of it from the start of an
 * asynchronous launch's admission work (state scatter, right-hand-side gather, column init) to its
 * step; ms3[2]: host time finishes spent after their step had drained.  No reference counterpart. */
int sg_engine_idle_ms(sg_ctx *ctx, double *ms3);
int sg_engine_reset_timing(sg_ctx *ctx);
/* Per-step records since the last sg_engine_reset_timing (at most 65536 steps), eight doubles each:
 * columns the GRM.V computed (active columns padded to its tile width), occupied columns, GRM.V
 * device ms, step device ms, device idle ms before the step (-1 for the first), host ms from the
 * previous step's finish to this step's launch (-1 for the first), host ms inside the launch, and
 * the slot uploads its admission waited for.  Up to max_steps records into out[8 * max_steps];
 * *n_out gets the count.  No reference counterpart. */
int sg_engine_step_trace(sg_ctx *ctx, double *out, int64_t max_steps, int64_t *n_out);
/* Bytes copied host->device and device->host by the engine calls (right-hand sides, weights,
 * probe tables, column states, fetched results, probe reductions) since the last
 * sg_engine_reset_timing.  No reference counterpart (I/O accounting of this engine). */
int sg_engine_io_bytes(sg_ctx *ctx, uint64_t *h2d_bytes, uint64_t *d2h_bytes);

/* ------------------------------------------------------------ synthetic cohorts (benchmarks / tests)
 * Writes a SNP-major .bed image (with magic) for n samples x m markers into device memory owned by
 * the context: p_m ~ U(0.01,0.5) by marker hash, HWE genotypes, missing with probability miss_rate.
 * The exact integer recipe is documented in saigegpu/synth.py and reproduced there on the CPU. */
int sg_synth_bed(sg_ctx *ctx, uint64_t seed, int64_t n, int64_t m, double miss_rate,
                 uint8_t **bed_dev, uint64_t *bed_len);
int sg_synth_bed_to_host(sg_ctx *ctx, uint8_t *host, uint64_t len);
/* g = Z b / sqrt(M_qc) with b_m ~ N(0,1) from the counter hash (polygenic signal). */
int sg_synth_genetic_value(sg_ctx *ctx, uint64_t seed, double *out);

/* ------------------------------------------------------------------ native batched fits
 * The null-model fit driver (glmmkin.ai_PCG_Rcpp_Binary / _Quantitative, FIT.R:79-549, with
 * Get_Coef, getCoefficients, getAIScore(_q), GetTrace(_q) and the fitglmmaiRPCG(_q) tau updates,
 * FIT.cpp:3113-3662) for many phenotypes at once over the engine, in native code.  No reference
 * counterpart as one call: the reference runs one phenotype per R process.
 *
 * sg_fits_create reserves the engine (max_columns; max_fits slots plus one spare per eight, at
 * most eight, where the next queued fits' subset set-ups run while they wait) and holds results on
 * the device; at most max_fits fits run at once.  sg_fits_submit queues a fit (admitted when
 * room and its columns are free): trait 0
 * binary (logit), 1 quantitative; mask is cohort-length (NULL = every sample) and y, X (n_sub x p,
 * column-major), offset (NULL = 0), eta0 and alpha0 are over the n_sub selected samples, as the R
 * driver's fit0.  sg_fits_run steps the engine until a fit finishes (or max_steps);
 * sg_fits_poll lists finished fits; sg_fits_result copies one out (theta 2, alpha p, eta / mu /
 * Y n_sub, cov p x p) and releases it, returning the fit's own error status if it failed
 * (message in sg_fits_last_error). */
typedef struct sg_fits sg_fits;
int sg_fits_create(sg_ctx *ctx, int64_t max_columns, int64_t max_fits, int pipelined, sg_fits **out);
void sg_fits_destroy(sg_fits *fits);
const char *sg_fits_last_error(sg_fits *fits);
int sg_fits_submit(sg_fits *fits, int trait, int64_t n_sub, const uint8_t *mask, const double *y,
                   const double *X, int p, const double *offset, const double *eta0, const double *alpha0,
                   double tol, int maxiter, int nrun, double tol_pcg, int maxiter_pcg, double cv_cutoff,
                   uint64_t seed, int64_t *fit_id);
int sg_fits_run(sg_fits *fits, int64_t max_steps, int64_t *n_ready);
/* Host threads for the fits' arithmetic; engine calls stay serialised.  threads > 1 (pipelined
 * drivers): threads - 1 workers resume fits while the calling thread steps the engine, launching
 * each step as soon as the last one has run, and sg_fits_run may return with workers still
 * resuming fits.  threads = 1: the calling thread alternates stepping and resuming.  Default: half
 * the hardware threads, at most 8. */
int sg_fits_set_threads(sg_fits *fits, int threads);
/* With worker threads: after a step finishes, the next launch waits up to ms (0..1000, default 0)
 * for the workers to resume the fits that step made ready, so that their new columns ride the
 * next step instead of the one after it (fewer steps per fit, at the cost of device idle time). */
int sg_fits_set_launch_wait(sg_fits *fits, double ms);
int sg_fits_poll(sg_fits *fits, int64_t *ids, int64_t max_ids, int64_t *n_out);
int sg_fits_counts(sg_fits *fits, int64_t *active, int64_t *pending, int64_t *done);
/* t8: seconds in engine steps (launch / finish / poll, and with worker threads the wait for the
 * step), seconds of driver work (summed over the worker threads when there are any), steps, the
 * parts of the driver work spent in weight uploads, submissions, result copies and probe
 * reductions, and the part of the engine time spent launching steps */
int sg_fits_host_times(sg_fits *fits, double *t8);
/* t4: with worker threads, seconds of the stepping thread's engine time spent waiting for the
 * step on the device, waiting for the driver's lock (a worker's engine call in progress),
 * finishing the step, and marking finished requests done. */
int sg_fits_step_times(sg_fits *fits, double *t4);
/* t3: for a finished fit not yet collected by sg_fits_result, the seconds since sg_fits_create at
 * which it was added, given a phenotype slot (admitted), and finished. */
int sg_fits_fit_times(sg_fits *fits, int64_t fit_id, double *t3);
int sg_fits_result(sg_fits *fits, int64_t fit_id, double *theta, double *alpha, double *eta, double *mu,
                   double *Y, double *cov, int32_t *iterations, int32_t *converged,
                   int64_t *column_iterations);

#ifdef __cplusplus
}
#endif
#endif /* SAIGEGPU_H */
