// C ABI of libsaigegpu (include/saigegpu.h): context, genotype set-up, GRM
// build, the continuous-batching PCG engine and the drop-ins for the
// reference's Rcpp entry points.  Host-side arithmetic that the reference does
// with Armadillo on p x p matrices (inverse of X' Sigma^-1 X, the 2x2 AI
// solve, tau updates) and the O(n) combinations around the solves run here in
// FP64; everything O(n^2) or larger runs in the CUDA kernels.
#include "sg_internal.h"
#include "host_math.h"
#include "../../include/saigegpu.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <fstream>
#include <string>
#include <unordered_map>
#include <vector>

using namespace sg;

namespace {

// set-up streams (lowest priority): slot s uses number s % kSetupStreams
constexpr int kSetupStreams = 4;

struct Req {
  int64_t id = 0;
  int64_t slot = 0;
  int kind = 0;       // 0 PCG, 1 product
  int maxiter = 0;
  double tol = 0.0;
  bool probe = false;
  uint64_t seed = 0;
  int64_t run = 0;
  double* b = nullptr;        // right-hand side in a pinned slab until admission copies it up
  const double* bd = nullptr; // the slab's device address (mapped pinned memory)
  int state = 0;      // 0 queued, 1 running, 2 done
  int64_t col = -1;
  std::vector<double> x;
  int32_t iters = 0;
  int64_t src = -1;   // chained: the right-hand side is this request's result (admitted once it is done)
};

struct Engine {
  int64_t cap_cols = 0, cap_ph = 0, np = 0, nblk = 0, stage_cols = 0;
  double *X = nullptr, *R = nullptr, *Z = nullptr, *P = nullptr, *B = nullptr, *part = nullptr;
  double *winv = nullptr, *minv = nullptr, *Yd = nullptr;
  float *Pf = nullptr, *Yf = nullptr;
  ColState* d_st = nullptr;
  PhenoState* d_ph = nullptr;
  int32_t* d_cols = nullptr;
  std::vector<ColState> h_st;
  std::vector<int64_t> col_req;
  std::vector<PhenoState> h_ph;
  std::vector<char> ph_set;
  std::deque<int64_t> queue;
  std::unordered_map<int64_t, Req> reqs;
  std::unordered_multimap<int64_t, int64_t> deps;  // source request -> chained requests still queued
  int64_t next_id = 1;
  int64_t hi_col = 0;
  int64_t n_active = 0;
  int64_t steps = 0, retired = 0, col_iters = 0, grm_passes = 0;
  std::vector<int64_t> finished;  // ids retired since the last poll
  bool hold = false;              // keep finished results on the device until fetched/consumed
  uint64_t io_h2d = 0, io_d2h = 0;  // bytes through the engine API since the last timing reset
  ColState* h_pin = nullptr;      // pinned mirror for the asynchronous state read-back of a step
  int32_t* h_gcols = nullptr;     // pinned: the step's active columns (GRM.V compaction, vector kernels)
  int64_t nact = 0;
  // pinned staging: column states for one scatter launch (h_sst / h_scol, n_sst staged), the
  // admitted columns and probe tables of an admission round, and slabs holding queued
  // right-hand sides; all copied up asynchronously
  ColState* h_sst = nullptr;
  int32_t* h_scol = nullptr;
  ColState* d_sst = nullptr;
  int32_t* d_scol = nullptr;
  int64_t n_sst = 0;
  std::vector<int32_t> stage_idx;  // column -> its entry in the current staging batch, or -1
  std::vector<int64_t> slab_pending;  // admitted requests whose slabs return once the stream drains
  int32_t* h_acols = nullptr;
  unsigned char* h_ptab = nullptr;
  std::vector<std::pair<double*, const double*>> slab_free;  // (pinned host, device) slab pairs
  std::vector<void*> slab_blocks;   // pinned host blocks
  std::vector<void*> slab_dblocks;  // device blocks
  cudaEvent_t ev_up = nullptr;      // the last right-hand-side upload (upload stream)
  bool up_wait = false;             // the next admission waits for it
  double* d_wstage[kSetupStreams] = {};  // their device copy (np doubles + np bytes), per set-up stream
  double* d_wstage2 = nullptr;    // the same for weight-only uploads (weights stream)
  int32_t* d_gcols = nullptr;
  bool inflight = false;          // a launched step has not been finished yet
  int64_t inflight_ncols = 0, inflight_occupied = 0, inflight_hi = 0;
  std::vector<int64_t> pending_release;  // columns freed on the host, reset on the device at the next launch
  float* Pflo = nullptr;          // low TF32 halves of Pf (split-TF32 mode)
  void* Pb = nullptr;             // BF16 high (first cap_cols * np) and low halves of Pf (split-BF16 mode)
  double* d_sx = nullptr;         // probe_dots: Sigma^-1 X block
  double* d_dpart = nullptr;      // probe_dots: block partial sums
  int32_t* d_dcols = nullptr;     // probe_dots: column indices
  uint8_t* ptab = nullptr;        // probe table of one admission round (stage_cols x 24 B)
  // K u of each slot's probes, kept between AI-REML iterations (the probes and the slot's sample
  // mask do not change during a fit): kProbeCache vectors per slot, keyed by (seed, run)
  double* pcache = nullptr;
  std::vector<std::vector<std::pair<uint64_t, int64_t>>> pcache_key;  // per slot: (seed, run) per entry
  size_t dots_cap_sx = 0, dots_cap_part = 0, dots_cap_cols = 0;
  // a probe reduction launched and not yet ended, per slot (sg_engine_probe_dots_begin / _end)
  struct DotsPending {
    bool pending = false;
    std::vector<int64_t> ids_pcg, ids_prod;
    int64_t k = 0, nv = 0, nblk = 0;
    double* h_part = nullptr;  // pinned block partials, k x nblk x nv
    size_t cap = 0;
    cudaEvent_t ev = nullptr;
  };
  std::vector<DotsPending> dots;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  cudaEvent_t ev_prev[3] = {nullptr, nullptr, nullptr};  // the previous step's (swapped per launch)
  bool have_prev = false;  // ev_prev holds a finished step whose end the idle time counts from
  double t_idle_ms = 0.0;  // device time between consecutive steps
  double t_admit_ms = 0.0; // of which: admission work queued at the launch (state scatter, RHS gather, init)
  double t_finish_host_ms = 0.0;  // host time a finish spends after the step has drained
  cudaEvent_t ev_adm = nullptr;
  bool adm_recorded = false;
  // host side of the step in flight: ms from the previous finish's return to its launch, ms inside
  // the launch, slot uploads its admission waited for
  std::chrono::steady_clock::time_point t_fin_end;
  bool have_fin_end = false;
  double inflight_gap_ms = -1.0, inflight_launch_ms = 0.0;
  int adm_waits = 0, inflight_waits = 0;
  // set_pheno uploads without waiting, through the slot's own pinned staging; ev_slot marks the end
  // of the slot's upload (and of any set-up before it on the set-up stream).  Columns of a slot whose
  // upload has not finished wait for it at admission, or stay queued for a later step when other
  // columns run meanwhile
  std::vector<double*> h_wslot;      // per slot: W (np doubles) then the mask (np bytes), pinned
  std::vector<cudaEvent_t> ev_slot;
  std::vector<uint8_t> slot_rec;     // ev_slot recorded at least once
  std::vector<uint8_t> slot_wait;    // the next admission of the slot's columns checks ev_slot
  double t_step_ms = 0, t_gemm_ms = 0, gemm_launches = 0, gemm_flops = 0, gemm_cols = 0, useful_cols = 0;
  // per-step records since the last timing reset (the first kStepTrace steps):
  // [columns the GRM.V computed, occupied columns, GRM.V ms, step ms, idle ms before the step]
  std::vector<double> trace;
  // subset-exact engine: per slot, the state of its sample subset (kept while the mask is the same)
  struct SlotSub {
    bool valid = false;
    bool all = false;             // built for "every sample" (no mask)
    std::vector<uint8_t> mask;    // the mask it was built for
    int64_t ex_lo = 0, ex_hi = -1;  // and the .bim markers it left out (a chromosome, or none)
    float* dp = nullptr;          // mg: d' = 1/sd'^2 (0 off the subset's GRM markers)
    float* p2 = nullptr;          // mg: 2p'
    float* lut = nullptr;         // mg x 4: d' (g - 2p')^2 per packed code (diagonal)
    int32_t* flips = nullptr;     // fill-changed markers (room for every marker)
    float* dfill = nullptr;
    uint32_t* bits = nullptr;     // W x np bit map (word-major)
    int64_t bits_cap = 0;
    double* diag = nullptr;       // np: sum of z'^2 (the preconditioner's diagonal)
    SubsetSlot dev;               // what d_slots[slot] holds
    double m_prime = 0.0;
    // first half of a set-up launched ahead (sg_engine_prepare_subset): QC records, flags and
    // counts of the subset in prep_mask, complete when ev_prep has
    MarkerQC* qc = nullptr;       // m_bim
    uint8_t* flag = nullptr;      // mg
    uint32_t* mb = nullptr;       // the mask as 2-bit fields
    // pinned staging of the mask fields and of the slot's device record: a copy from pageable
    // memory may wait for the work queued before it on the (low-priority) set-up stream
    uint32_t* h_mb = nullptr;
    SubsetSlot* h_rec = nullptr;
    int64_t* d_counts = nullptr;  // (changes, M')
    int64_t* h_counts = nullptr;  // pinned copy
    cudaEvent_t ev_prep = nullptr;
    bool prep = false;
    bool prep_all = false;
    std::vector<uint8_t> prep_mask;
    int64_t prep_ns = 0;
    int64_t prep_lo = 0, prep_hi = -1;
  };
  std::vector<SlotSub> sub;
  SubsetSlot* d_slots = nullptr;
  int max_w = 0;
  void* Vb = nullptr;             // centred P halves: cap_cols x np BF16, high then low
  float* Tm = nullptr;            // T = G^T v_c: cap_cols x mg
  void* Tb = nullptr;             // T' halves: cap_cols x mg BF16, high then low
  float* Um = nullptr;            // U = G T': cap_cols x np
  double* spart = nullptr;        // column partials: cap_cols x max(blocks over np, over mg)
  float* smax = nullptr;          // FP16 / E4M3 form: column block maxima, as spart
  float* sscale = nullptr;        //   and the columns' power-of-two scales s1, s2 (2 x cap_cols)
  float* sdiag_part[kSetupStreams] = {};  // per-chunk partial sums of a subset's diagonal, per set-up stream

};
constexpr int64_t kStepTrace = 65536;
constexpr int kTraceFields = 8;

}  // namespace

struct sg_ctx {
  int device = 0;
  uint64_t budget = 0;
  uint64_t in_use = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t side = nullptr;  // result copies and probe reductions overlap a step here
  cudaStream_t up = nullptr;    // the engine's right-hand-side uploads
  // phenotype slots' set-ups (subset QC and tables, first weights): slot s on setup[s % kSetupStreams],
  // so that a slot's set-up waits only for the set-ups queued before it on its own stream
  cudaStream_t setup[kSetupStreams] = {};
  cudaStream_t wts = nullptr;    // later weight uploads of slots already set up
  std::string err;
  std::string err_pending;
  uint64_t launches = 0;
  int mv_mode = SG_MV_FP32_SIMT;
  std::unordered_map<void*, size_t> allocs;
  // genotypes
  bool have_geno = false;
  int64_t n_fam = 0, m_bim = 0, nn = 0, m_qc = 0, m_vr = 0, pitch = 0;
  int is_diag_one = 0;
  uint8_t* d_packed = nullptr;
  uint8_t* d_packed_vr = nullptr;
  float* d_lut = nullptr;
  float* d_lut_vr = nullptr;
  std::vector<float> freq, invstd, vr_freq;
  std::vector<int32_t> mac, vr_mac, vr_index;
  std::vector<uint8_t> qc_mask;
  // GRM
  bool have_grm = false;
  int64_t np = 0;
  float* d_K = nullptr;
  float* d_Klo = nullptr;   // K - tf32(K) while the split-TF32 engine is selected (d_K then holds tf32(K))
  bool k_split = false;
  int num_sms = 152;
  int diag_frac_bits = 32;  // fixed-point scale of the high-precision diagonal
  void* d_Kb = nullptr;     // BF16 high (first n_p^2) and low halves of K for SG_MV_BF16X3_TC
  double* d_diag = nullptr;
  float* d_diag32 = nullptr;
  std::vector<double> diag;
  std::vector<float> diag32;
  // leave-one-chromosome-out state (setStartEndIndex, FIT.cpp:3067-3085)
  bool loco = false;
  int64_t loco_begin = 0, loco_end = -1, loco_mj = 0, loco_mjp = 0;
  float* d_zm = nullptr;   // Z_j marker-major (mjp x np)
  float* d_zs = nullptr;   // Z_j sample-major (np x mjp)
  float* d_lu = nullptr;   // Z_j' P  (cap_cols x mjp)
  float* d_lv = nullptr;   // Z_j Z_j' P (cap_cols x np)
  float* d_lp = nullptr;   // P in full FP32 for the correction (cap_cols x np)
  std::vector<double> diag_loco;
  double* d_diag_loco = nullptr;  // its device copy (slot weights)
  // the subset-exact engines: .bim markers sub_loco_lo..sub_loco_hi left out of every phenotype's
  // GRM (none when lo > hi); each slot's subset state is rebuilt for it at the slot's next set
  int64_t sub_loco_lo = 0, sub_loco_hi = -1;
  // device time of the last setgeno ([0] QC, [1] re-pack + LUT, [2] diagonal) and grm_build
  // ([3] Z build, [4] SYRK), in ms, from CUDA events on the context stream
  double t_build[5] = {0, 0, 0, 0, 0};
  cudaEvent_t tev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  // every .bim marker in cohort order with missing calls kept, the cohort fill and the
  // variance-ratio candidates per .bim marker, and setgeno's thresholds: what the subset-exact
  // engine recomputes a phenotype subset's QC from
  uint8_t* d_codes = nullptr;
  uint8_t* d_vrflag_all = nullptr;
  int32_t* d_fill_all = nullptr;  // the cohort fill of every .bim marker (subset-exact engine)
  std::vector<int32_t> fill_all;
  float qc_min_maf = 0.01f, qc_max_missing = 0.15f, qc_min_mac_vr = 20.0f, qc_max_mac_vr = -1.0f;
  // upper MAC bound of categorical variance ratios for the next setgeno (-1: a single ratio)
  float vr_max_mac = -1.0f;
  int qc_is_var_ratio = 0;
  // subset-exact engine: genotype values 0/1/2 (cohort fill in missing calls) in BF16, marker-major
  // (mg x np) then sample-major (np x mg), mg = .bim markers rounded up to 128
  void* d_G = nullptr;   // genotype matrix: BF16 (form 0) or FP16 then E4M3 (form 1), both layouts each
  int g_form = 0;
  int64_t mg = 0;
  // synthetic bed image
  uint8_t* d_synth = nullptr;
  uint64_t synth_len = 0;
  Engine eng;
};

// ------------------------------------------------------------------ helpers
extern "C" int sg_engine_probe_dots(sg_ctx* c, int64_t slot, const int64_t* ids_pcg,
                                    const int64_t* ids_prod, int64_t k, uint64_t seed, int64_t run0,
                                    const double* SX, int64_t p, double* out, int32_t* iters);

static float ev_ms(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

static int set_err(sg_ctx* c, int code, const char* fmt, ...) {
  if (!c) return code;
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  c->err = buf;
  return code;
}

#define SG_CUDA(c, call)                                                                  \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return set_err((c), SG_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

#define SG_LAUNCHED(c, n)                                                                     \
  do {                                                                                        \
    (c)->launches += (n);                                                                     \
    cudaError_t e_ = cudaGetLastError();                                                      \
    if (e_ != cudaSuccess) return set_err((c), SG_ERR_CUDA, "kernel launch: %s", cudaGetErrorString(e_)); \
  } while (0)

#define SG_TRY(x)            \
  do {                       \
    int r_ = (x);            \
    if (r_ != SG_OK) return r_; \
  } while (0)

static int dev_alloc(sg_ctx* c, void** p, size_t bytes) {
  *p = nullptr;
  if (bytes == 0) bytes = 16;
  if (c->budget && c->in_use + bytes > c->budget)
    return set_err(c, SG_ERR_NOMEM, "HBM budget exceeded: %zu + %zu > %llu", (size_t)c->in_use,
                   bytes, (unsigned long long)c->budget);
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    return set_err(c, SG_ERR_NOMEM, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
  }
  c->allocs[*p] = bytes;
  c->in_use += bytes;
  return SG_OK;
}

template <typename T>
static int dev_alloc_t(sg_ctx* c, T** p, size_t count) {
  return dev_alloc(c, reinterpret_cast<void**>(p), count * sizeof(T));
}

static void dev_free(sg_ctx* c, void* p) {
  if (!p) return;
  auto it = c->allocs.find(p);
  if (it != c->allocs.end()) {
    c->in_use -= it->second;
    c->allocs.erase(it);
  }
  cudaFree(p);
}
template <typename T>
static void dev_free_t(sg_ctx* c, T*& p) {
  dev_free(c, (void*)p);
  p = nullptr;
}

static int sync(sg_ctx* c) {
  SG_CUDA(c, cudaStreamSynchronize(c->stream));
  return SG_OK;
}

static int sync_side(sg_ctx* c) {
  SG_CUDA(c, cudaStreamSynchronize(c->side));
  return SG_OK;
}

// Host<->device copies of the engine API, counted for its I/O report (sg_engine_io_bytes).
static cudaError_t h2d(sg_ctx* c, void* dst, const void* src, size_t bytes, cudaStream_t s);
static cudaError_t d2h(sg_ctx* c, void* dst, const void* src, size_t bytes, cudaStream_t s);

static bool all_finite(const float* v, int64_t n) {
  for (int64_t i = 0; i < n; ++i)
    if (!std::isfinite(v[i])) return false;
  return true;
}
static bool all_finite(const double* v, int64_t n) {
  for (int64_t i = 0; i < n; ++i)
    if (!std::isfinite(v[i])) return false;
  return true;
}

// ------------------------------------------------------------------ context
extern "C" int sg_ctx_create(int device, uint64_t hbm_budget_bytes, sg_ctx** out) {
  if (!out) return SG_ERR_INVALID;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= device || device < 0) {
    cudaGetLastError();
    return SG_ERR_CUDA;
  }
  if (cudaSetDevice(device) != cudaSuccess) return SG_ERR_CUDA;
  sg_ctx* c = new sg_ctx();
  c->device = device;
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (c->num_sms <= 0) c->num_sms = 1;
  c->budget = hbm_budget_bytes;
  // Three priorities (numerically lower is dispatched first).  The side stream carries short
  // reductions and copies that the driver waits on while a step's GEMM fills the GPU: highest, so
  // its blocks are dispatched as soon as an SM frees up.  The steps run above the slots' set-ups,
  // whose blocks then fill the SMs a step leaves idle (the last wave of each GEMM, the short kernels
  // between them) instead of taking SMs from the GEMMs.
  int prio_lo = 0, prio_hi = 0;
  cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
  const int prio_step = prio_lo > prio_hi ? prio_lo - 1 : prio_lo;
  if (cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, prio_step) != cudaSuccess) {
    delete c;
    return SG_ERR_CUDA;
  }
  for (auto& ev : c->tev) cudaEventCreate(&ev);
  if (cudaStreamCreateWithPriority(&c->side, cudaStreamNonBlocking, prio_hi) != cudaSuccess) {
    cudaStreamDestroy(c->stream);
    delete c;
    return SG_ERR_CUDA;
  }
  for (auto& st : c->setup)
    if (cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, prio_lo) != cudaSuccess) {
      for (auto& x : c->setup)
        if (x) cudaStreamDestroy(x);
      cudaStreamDestroy(c->side);
      cudaStreamDestroy(c->stream);
      delete c;
      return SG_ERR_CUDA;
    }
  // a slot's new weights (every AI-REML iteration) must not queue behind other slots' set-ups
  if (cudaStreamCreateWithPriority(&c->wts, cudaStreamNonBlocking, prio_hi) != cudaSuccess) {
    for (auto& x : c->setup) cudaStreamDestroy(x);
    cudaStreamDestroy(c->side);
    cudaStreamDestroy(c->stream);
    delete c;
    return SG_ERR_CUDA;
  }
  // right-hand-side uploads of the engine, beside the steps (copy engine only)
  if (cudaStreamCreateWithFlags(&c->up, cudaStreamNonBlocking) != cudaSuccess) {
    cudaStreamDestroy(c->wts);
    for (auto& x : c->setup) cudaStreamDestroy(x);
    cudaStreamDestroy(c->side);
    cudaStreamDestroy(c->stream);
    delete c;
    return SG_ERR_CUDA;
  }
  *out = c;
  return SG_OK;
}

static void engine_free(sg_ctx* c);

extern "C" void sg_ctx_destroy(sg_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  cudaStreamSynchronize(c->side);
  for (auto& x : c->setup) cudaStreamSynchronize(x);
  cudaStreamSynchronize(c->wts);
  cudaStreamSynchronize(c->up);
  engine_free(c);  // the engine's device buffers, pinned staging and events
  for (auto& kv : c->allocs) cudaFree(kv.first);
  c->allocs.clear();
  cudaStreamDestroy(c->up);
  cudaStreamDestroy(c->wts);
  for (auto& x : c->setup) cudaStreamDestroy(x);
  cudaStreamDestroy(c->side);
  cudaStreamDestroy(c->stream);
  delete c;
}

extern "C" const char* sg_last_error(const sg_ctx* c) { return c ? c->err.c_str() : "null context"; }

extern "C" int sg_device_bytes_in_use(const sg_ctx* c, uint64_t* bytes) {
  if (!c || !bytes) return SG_ERR_INVALID;
  *bytes = c->in_use;
  return SG_OK;
}

__global__ void add_inplace_kernel(float* a, const float* b, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = a[i] + b[i];
}

static int ensure_k_split(sg_ctx* c, bool want);
static int ensure_k_bf16(sg_ctx* c, bool want);
static void engine_free(sg_ctx* c);

static int ensure_g(sg_ctx* c, int form);

// the subset-exact engines (BF16 products, or FP16 high / E4M3 low)
static bool exact_mode(int mode) { return mode == SG_MV_SUBSET_EXACT || mode == SG_MV_SUBSET_EXACT_F8; }

extern "C" int sg_set_matvec_mode(sg_ctx* c, int mode) {
  if (!c) return SG_ERR_INVALID;
  if (mode != SG_MV_FP32_SIMT && mode != SG_MV_TF32_TC && mode != SG_MV_FP64_PLAIN &&
      mode != SG_MV_TF32X3_TC && mode != SG_MV_BF16X3_TC && !exact_mode(mode))
    return set_err(c, SG_ERR_INVALID, "unknown matvec mode %d", mode);
  if ((mode == SG_MV_TF32_TC || mode == SG_MV_TF32X3_TC || mode == SG_MV_BF16X3_TC || exact_mode(mode)) &&
      !tc_available())
    return set_err(c, SG_ERR_INVALID, "tcgen05 path needs an sm_103a device");
  if (c->eng.inflight) return set_err(c, SG_ERR_STATE, "a step is in flight: finish it first");
  if (exact_mode(mode)) {
    if (!c->have_geno) return set_err(c, SG_ERR_STATE, "setgeno has not run");
    if (c->loco) return set_err(c, SG_ERR_STATE, "clear the LOCO range first (sg_loco_clear)");
    for (auto& kv : c->eng.reqs)
      if (kv.second.state == 1) return set_err(c, SG_ERR_STATE, "columns in flight");
  } else if (c->sub_loco_lo <= c->sub_loco_hi) {
    return set_err(c, SG_ERR_STATE, "clear the LOCO range first (sg_loco_clear)");
  }
  const bool was_exact = exact_mode(c->mv_mode);
  c->mv_mode = mode;
  // a slot's subset state and preconditioner belong to the engine they were set for: entering or
  // leaving the subset-exact engines asks for every slot to be set again (the two forms share it)
  if (was_exact != exact_mode(mode)) {
    for (auto& ss : c->eng.sub) {
      if (ss.prep) cudaEventSynchronize(ss.ev_prep);
      ss.valid = ss.prep = false;
    }
    std::fill(c->eng.ph_set.begin(), c->eng.ph_set.end(), 0);
  }
  if (exact_mode(mode)) {
    SG_TRY(ensure_k_split(c, false));
    SG_TRY(ensure_k_bf16(c, false));
    return ensure_g(c, mode == SG_MV_SUBSET_EXACT_F8 ? 1 : 0);
  }
  if (was_exact) {  // the genotype matrix (2 bytes per sample and marker, twice) leaves HBM
    SG_TRY(sync(c));
    dev_free(c, c->d_G);
    c->d_G = nullptr;
  }
  if (!c->have_grm) return SG_OK;
  SG_TRY(ensure_k_split(c, mode == SG_MV_TF32X3_TC));
  return ensure_k_bf16(c, mode == SG_MV_BF16X3_TC);
}

// Genotype values of every .bim marker for the subset-exact engines, both layouts: in BF16 (form 0),
// or in FP16 and in E4M3 (form 1); all exact.
static int ensure_g(sg_ctx* c, int form) {
  if (c->d_G && c->g_form == form) return SG_OK;
  if (c->d_G) {  // the other form's matrix leaves HBM first
    SG_TRY(sync(c));
    dev_free(c, c->d_G);
    c->d_G = nullptr;
  }
  const int64_t np = round_up(c->nn, kRowTile), mg = round_up(std::max<int64_t>(c->m_bim, 1), kRowTile);
  if (c->have_grm && c->np != np) return set_err(c, SG_ERR_STATE, "GRM row padding differs");
  if (!c->have_grm) {
    engine_free(c);
    c->np = np;
  }
  // the cohort fill stays on the device beside G: each subset's set-up compares its own fill with it
  if (!c->d_fill_all) SG_TRY(dev_alloc_t(c, &c->d_fill_all, (size_t)std::max<int64_t>(c->m_bim, 1)));
  SG_TRY(dev_alloc(c, &c->d_G, (size_t)(2 * mg * np * (form ? 3 : 2))));
  c->g_form = form;
  if (c->m_bim)
    SG_CUDA(c, cudaMemcpyAsync(c->d_fill_all, c->fill_all.data(), c->m_bim * 4, cudaMemcpyHostToDevice, c->stream));
  SG_CUDA(c, cudaEventRecord(c->tev[0], c->stream));
  uint16_t* g16 = static_cast<uint16_t*>(c->d_G);
  uint8_t* g8 = reinterpret_cast<uint8_t*>(g16 + 2 * mg * np);
  launch_gbuild(c->d_codes, c->pitch, c->d_fill_all, c->m_bim, c->nn, mg, np, form, g16, g16 + mg * np,
                form ? g8 : nullptr, form ? g8 + mg * np : nullptr, c->stream);
  SG_LAUNCHED(c, 1);
  SG_CUDA(c, cudaEventRecord(c->tev[1], c->stream));
  SG_TRY(sync(c));
  c->t_build[3] = ev_ms(c->tev[0], c->tev[1]);
  c->mg = mg;
  return SG_OK;
}

extern "C" int sg_ctx_make_current(sg_ctx* c) {
  if (!c) return SG_ERR_INVALID;
  SG_CUDA(c, cudaSetDevice(c->device));
  return SG_OK;
}

extern "C" int sg_selftest_wait_timeout(sg_ctx* c, double budget_ms) {
  if (!c) return SG_ERR_INVALID;
  if (budget_ms <= 0 || budget_ms > 2000) return set_err(c, SG_ERR_INVALID, "budget must be in (0, 2000] ms");
  int waited_out = 0;
  cudaError_t e = tc_wait_selftest(budget_ms, &waited_out, c->stream);
  c->launches += 1;
  if (e == cudaErrorLaunchTimeout && waited_out)
    return set_err(c, SG_ERR_TIMEOUT, "bounded device wait gave up after %.1f ms", budget_ms);
  if (e != cudaSuccess) return set_err(c, SG_ERR_CUDA, "self-test: %s", cudaGetErrorString(e));
  return set_err(c, SG_ERR_STATE, "the wait completed although nothing arrived");
}

extern "C" int sg_set_tc_option(sg_ctx* c, int option, int value) {
  if (!c) return SG_ERR_INVALID;
  if (!tc_set_option(option, value))
    return set_err(c, SG_ERR_INVALID, "tcgen05 option %d cannot take the value %d", option, value);
  return SG_OK;
}

extern "C" int sg_get_tc_option(sg_ctx* c, int option, int* value) {
  if (!c || !value) return SG_ERR_INVALID;
  const int v = tc_get_option(option);
  if (v < 0) return set_err(c, SG_ERR_INVALID, "unknown tcgen05 option %d", option);
  *value = v;
  return SG_OK;
}

extern "C" int sg_set_grmv_plan(sg_ctx* c, int n, const int32_t* max_cols, const int32_t* pair,
                                const int32_t* slice) {
  if (!c || n < 0 || n > 64 || (n > 0 && (!max_cols || !pair || !slice))) return SG_ERR_INVALID;
  if (!tc_set_grmv_plan(max_cols, pair, slice, n))
    return set_err(c, SG_ERR_INVALID, "plan buckets need increasing max_cols, pair 0/1 and slice 0/64/128");
  return SG_OK;
}

extern "C" int sg_get_grmv_plan(sg_ctx* c, int cap, int32_t* max_cols, int32_t* pair, int32_t* slice,
                                int* n) {
  if (!c || !n || cap < 0 || (cap > 0 && (!max_cols || !pair || !slice))) return SG_ERR_INVALID;
  *n = tc_get_grmv_plan(max_cols, pair, slice, cap);
  return SG_OK;
}

extern "C" int sg_set_vr_max_mac(sg_ctx* c, float max_mac) {
  if (!c) return SG_ERR_INVALID;
  if (max_mac != -1.0f && !(max_mac > 0.0f)) return set_err(c, SG_ERR_INVALID, "max MAC must be -1 or positive");
  c->vr_max_mac = max_mac;
  return SG_OK;
}

extern "C" int sg_set_subset_plan(sg_ctx* c, int n, const int32_t* max_cols, const int32_t* pair,
                                  const int32_t* slice) {
  if (!c || n < 0 || n > 64 || (n > 0 && (!max_cols || !pair || !slice))) return SG_ERR_INVALID;
  if (!tc_set_subset_plan(max_cols, pair, slice, n))
    return set_err(c, SG_ERR_INVALID, "plan buckets need increasing max_cols, pair 0/1 and slice 64/128");
  return SG_OK;
}

extern "C" int sg_get_subset_plan(sg_ctx* c, int cap, int32_t* max_cols, int32_t* pair, int32_t* slice, int* n) {
  if (!c || !n || cap < 0 || (cap > 0 && (!max_cols || !pair || !slice))) return SG_ERR_INVALID;
  *n = tc_get_subset_plan(max_cols, pair, slice, cap);
  return SG_OK;
}

extern "C" int sg_kernel_launches(const sg_ctx* c, uint64_t* count) {
  if (!c || !count) return SG_ERR_INVALID;
  *count = c->launches;
  return SG_OK;
}

// ------------------------------------------------------------------ genotypes
static void engine_free(sg_ctx* c);

static void loco_free(sg_ctx* c);

static void free_geno(sg_ctx* c) {
  engine_free(c);
  loco_free(c);
  c->sub_loco_lo = 0;
  c->sub_loco_hi = -1;
  dev_free_t(c, c->d_packed);
  dev_free_t(c, c->d_packed_vr);
  dev_free_t(c, c->d_lut);
  dev_free_t(c, c->d_lut_vr);
  dev_free_t(c, c->d_K);
  dev_free_t(c, c->d_Klo);
  c->k_split = false;
  dev_free(c, c->d_Kb);
  c->d_Kb = nullptr;
  dev_free_t(c, c->d_diag);
  dev_free_t(c, c->d_diag32);
  dev_free_t(c, c->d_codes);
  dev_free_t(c, c->d_vrflag_all);
  dev_free_t(c, c->d_fill_all);
  dev_free(c, c->d_G);
  c->d_G = nullptr;
  c->fill_all.clear();
  c->have_geno = false;
  c->have_grm = false;
}

// Fractional bits of the fixed-point diagonal: the largest F with m_qc * max z^2 * 2^F below
// 2^64 (a 1% margin), so no sample's sum can overflow.  z = (g - 2p) / sd per the LUT.
static int diag_frac_bits(const sg_ctx* c) {
  double zmax2 = 0.0;
  for (size_t j = 0; j < c->freq.size(); ++j) {
    const double p2 = 2.0 * (double)c->freq[j], s = (double)c->invstd[j];
    for (double g : {0.0, 1.0, 2.0}) zmax2 = std::max(zmax2, (g - p2) * (g - p2) * s * s);
  }
  const double bound = std::max(1.0, (double)c->freq.size() * zmax2 * 1.01);
  const int f = (int)std::floor(std::log2(18446744073709551615.0 / bound));
  return std::max(0, std::min(f, 62));
}

// raw: device .bed body re-pitched (m_bim rows of raw_pitch bytes, zero padded)
static int setgeno_core(sg_ctx* c, const uint8_t* raw, int64_t raw_pitch, int64_t n_fam,
                        int64_t m_bim, const int32_t* sub_1based, int64_t n_sub,
                        const uint8_t* pheno_mask, float min_maf, float max_missing,
                        const int32_t* vr_markers, int64_t n_vr, float min_mac_vr,
                        int is_var_ratio, int is_diag_one) {
  const int64_t nn = n_sub;
  // pheno mask bits (bit 2s of word s/16) and the variance-ratio candidate flags
  const int64_t nwords = (n_fam + 15) / 16;
  std::vector<uint32_t> maskbits(nwords + 1, 0u);
  for (int64_t i = 0; i < n_fam; ++i)
    if (!pheno_mask || pheno_mask[i]) maskbits[i / 16] |= 1u << (2 * (i % 16));
  std::vector<uint8_t> vrflag(m_bim, 0);
  for (int64_t k = 0; k < n_vr; ++k) {
    if (vr_markers[k] < 0 || vr_markers[k] >= m_bim)
      return set_err(c, SG_ERR_INVALID, "variance-ratio marker index %d out of range", vr_markers[k]);
    vrflag[vr_markers[k]] = 1;
  }
  std::vector<int32_t> sub0(nn);
  bool identity = (nn == n_fam);
  for (int64_t k = 0; k < nn; ++k) {
    const int32_t s = sub_1based ? sub_1based[k] : (int32_t)(k + 1);
    if (s < 1 || s > n_fam) return set_err(c, SG_ERR_INVALID, "subSampleInGeno[%lld] = %d out of range", (long long)k, s);
    sub0[k] = s - 1;
    if (sub0[k] != k) identity = false;
  }
  uint32_t* d_mask = nullptr;
  uint8_t* d_vrflag = nullptr;
  MarkerQC* d_qc = nullptr;
  int32_t* d_sub = nullptr;
  SG_TRY(dev_alloc_t(c, &d_mask, maskbits.size()));
  SG_TRY(dev_alloc_t(c, &d_vrflag, (size_t)std::max<int64_t>(m_bim, 1)));
  SG_TRY(dev_alloc_t(c, &d_qc, (size_t)std::max<int64_t>(m_bim, 1)));
  SG_TRY(dev_alloc_t(c, &d_sub, (size_t)std::max<int64_t>(nn, 1)));
  SG_CUDA(c, cudaMemcpyAsync(d_mask, maskbits.data(), maskbits.size() * 4, cudaMemcpyHostToDevice, c->stream));
  if (m_bim) SG_CUDA(c, cudaMemcpyAsync(d_vrflag, vrflag.data(), m_bim, cudaMemcpyHostToDevice, c->stream));
  if (nn) SG_CUDA(c, cudaMemcpyAsync(d_sub, sub0.data(), nn * 4, cudaMemcpyHostToDevice, c->stream));
  SG_CUDA(c, cudaEventRecord(c->tev[0], c->stream));
  launch_marker_qc(raw, raw_pitch, m_bim, n_fam, d_mask, nn, min_maf, max_missing, d_vrflag,
                   min_mac_vr, c->vr_max_mac, is_var_ratio, d_qc, c->stream);
  SG_LAUNCHED(c, 1);
  SG_CUDA(c, cudaEventRecord(c->tev[1], c->stream));
  std::vector<MarkerQC> qc(m_bim);
  if (m_bim) SG_CUDA(c, cudaMemcpyAsync(qc.data(), d_qc, m_bim * sizeof(MarkerQC), cudaMemcpyDeviceToHost, c->stream));
  SG_TRY(sync(c));
  // marker compaction in .bim order (SNPIdx_new / SNPIdx_vr, FIT.cpp:900-947)
  std::vector<int32_t> src_qc, src_vr;
  c->freq.clear(); c->invstd.clear(); c->mac.clear(); c->qc_mask.assign(m_bim, 0);
  c->vr_freq.clear(); c->vr_mac.clear(); c->vr_index.clear();
  for (int64_t i = 0; i < m_bim; ++i) {
    if (qc[i].pass_qc) {
      src_qc.push_back((int32_t)i);
      c->freq.push_back(qc[i].freq);
      c->invstd.push_back(qc[i].invstd);
      c->mac.push_back(qc[i].mac);
      c->qc_mask[i] = 1;
    }
    if (qc[i].pass_vr) {
      src_vr.push_back((int32_t)i);
      c->vr_freq.push_back(qc[i].freq);
      c->vr_mac.push_back(qc[i].mac);
      c->vr_index.push_back((int32_t)i);
    }
  }
  c->fill_all.resize(m_bim);
  for (int64_t i = 0; i < m_bim; ++i) c->fill_all[i] = qc[i].fill;
  c->qc_min_maf = min_maf;
  c->qc_max_missing = max_missing;
  c->qc_min_mac_vr = min_mac_vr;
  c->qc_max_mac_vr = c->vr_max_mac;
  c->qc_is_var_ratio = is_var_ratio;
  c->nn = nn;
  c->n_fam = n_fam;
  c->m_bim = m_bim;
  c->m_qc = (int64_t)src_qc.size();
  c->m_vr = (int64_t)src_vr.size();
  c->is_diag_one = is_diag_one;
  c->pitch = round_up(std::max<int64_t>((nn + 3) / 4, 1), kPitchAlign);
  int32_t* d_src = nullptr;
  const int64_t nsrc = std::max<int64_t>(c->m_qc + c->m_vr, 1);
  SG_TRY(dev_alloc_t(c, &d_src, (size_t)nsrc));
  std::vector<int32_t> srcs(src_qc);
  srcs.insert(srcs.end(), src_vr.begin(), src_vr.end());
  if (!srcs.empty())
    SG_CUDA(c, cudaMemcpyAsync(d_src, srcs.data(), srcs.size() * 4, cudaMemcpyHostToDevice, c->stream));
  SG_TRY(dev_alloc_t(c, &c->d_packed, (size_t)std::max<int64_t>(c->m_qc * c->pitch, 16)));
  SG_TRY(dev_alloc_t(c, &c->d_packed_vr, (size_t)std::max<int64_t>(c->m_vr * c->pitch, 16)));
  SG_TRY(dev_alloc_t(c, &c->d_lut, (size_t)std::max<int64_t>(c->m_qc * 4, 4)));
  SG_TRY(dev_alloc_t(c, &c->d_lut_vr, (size_t)std::max<int64_t>(c->m_vr * 4, 4)));
  SG_CUDA(c, cudaEventRecord(c->tev[2], c->stream));
  launch_repack(raw, raw_pitch, d_src, d_qc, c->m_qc, d_sub, nn, identity ? 1 : 0, c->d_packed,
                c->pitch, c->stream);
  launch_repack(raw, raw_pitch, d_src + c->m_qc, d_qc, c->m_vr, d_sub, nn, identity ? 1 : 0,
                c->d_packed_vr, c->pitch, c->stream);
  launch_lut(d_qc, d_src, c->m_qc, c->d_lut, c->stream);
  launch_lut(d_qc, d_src + c->m_qc, c->m_vr, c->d_lut_vr, c->stream);
  SG_LAUNCHED(c, 4);
  SG_CUDA(c, cudaEventRecord(c->tev[3], c->stream));
  // every marker in cohort order with missing calls kept (the subset-exact engine's source)
  {
    std::vector<int32_t> all(m_bim);
    for (int64_t i = 0; i < m_bim; ++i) all[i] = (int32_t)i;
    int32_t* d_all = nullptr;
    SG_TRY(dev_alloc_t(c, &d_all, (size_t)std::max<int64_t>(m_bim, 1)));
    SG_TRY(dev_alloc_t(c, &c->d_codes, (size_t)std::max<int64_t>(m_bim * c->pitch, 16)));
    if (m_bim) SG_CUDA(c, cudaMemcpyAsync(d_all, all.data(), m_bim * 4, cudaMemcpyHostToDevice, c->stream));
    launch_repack(raw, raw_pitch, d_all, nullptr, m_bim, d_sub, nn, identity ? 1 : 0, c->d_codes, c->pitch,
                  c->stream);
    SG_LAUNCHED(c, 1);
    SG_TRY(sync(c));
    dev_free(c, d_all);
  }
  SG_TRY(sync(c));
  c->t_build[0] = ev_ms(c->tev[0], c->tev[1]);
  c->t_build[1] = ev_ms(c->tev[2], c->tev[3]);
  dev_free(c, d_src);
  dev_free(c, d_mask);
  c->d_vrflag_all = d_vrflag;  // kept for the subset-exact engine's per-subset QC
  dev_free(c, d_qc);
  dev_free(c, d_sub);
  // GRM diagonal from the packed genotypes
  SG_TRY(dev_alloc_t(c, &c->d_diag, (size_t)std::max<int64_t>(nn, 1)));
  SG_TRY(dev_alloc_t(c, &c->d_diag32, (size_t)std::max<int64_t>(nn, 1)));
  c->diag_frac_bits = diag_frac_bits(c);
  void* lutq = nullptr;  // per-marker tables of the diagonal
  SG_TRY(dev_alloc(c, &lutq, (size_t)std::max<int64_t>(48 * c->m_qc, 48)));
  SG_CUDA(c, cudaEventRecord(c->tev[0], c->stream));
  launch_diag(c->d_packed, c->pitch, c->d_lut, c->m_qc, nn, c->diag_frac_bits, lutq, c->d_diag,
              c->d_diag32, c->stream);
  SG_LAUNCHED(c, 2);
  SG_CUDA(c, cudaEventRecord(c->tev[1], c->stream));
  c->diag.resize(nn);
  c->diag32.resize(nn);
  if (nn) {
    SG_CUDA(c, cudaMemcpyAsync(c->diag.data(), c->d_diag, nn * 8, cudaMemcpyDeviceToHost, c->stream));
    SG_CUDA(c, cudaMemcpyAsync(c->diag32.data(), c->d_diag32, nn * 4, cudaMemcpyDeviceToHost, c->stream));
  }
  SG_TRY(sync(c));
  dev_free(c, lutq);
  c->t_build[2] = ev_ms(c->tev[0], c->tev[1]);
  c->have_geno = true;
  return SG_OK;
}

static int setgeno_common(sg_ctx* c, const uint8_t* bed, bool on_device, uint64_t bed_len,
                          int64_t n_fam, int64_t m_bim, const int32_t* sub_1based, int64_t n_sub,
                          const uint8_t* pheno_mask, float min_maf, float max_missing,
                          const int32_t* vr_markers, int64_t n_vr, float min_mac_vr,
                          int is_var_ratio, int is_diag_one) {
  if (!c) return SG_ERR_INVALID;
  if (!bed || n_fam <= 0 || m_bim < 0 || n_sub <= 0 || n_sub > n_fam || (n_vr > 0 && !vr_markers))
    return set_err(c, SG_ERR_INVALID, "setgeno: invalid arguments");
  const int64_t nb = (n_fam + 3) / 4;
  if (bed_len < (uint64_t)(3 + nb * m_bim))
    return set_err(c, SG_ERR_INVALID, "setgeno: .bed has %llu bytes, need %lld",
                   (unsigned long long)bed_len, (long long)(3 + nb * m_bim));
  uint8_t magic[3];
  if (on_device) {
    SG_CUDA(c, cudaMemcpy(magic, bed, 3, cudaMemcpyDeviceToHost));
  } else {
    memcpy(magic, bed, 3);
  }
  if (magic[0] != 0x6C || magic[1] != 0x1B || magic[2] != 0x01)
    return set_err(c, SG_ERR_INVALID, "setgeno: not a SNP-major PLINK .bed (magic %02x %02x %02x)",
                   magic[0], magic[1], magic[2]);
  free_geno(c);
  const int64_t raw_pitch = round_up(std::max<int64_t>(nb, 1), kPitchAlign);
  uint8_t* raw = nullptr;
  SG_TRY(dev_alloc_t(c, &raw, (size_t)std::max<int64_t>(raw_pitch * m_bim, 16)));
  SG_CUDA(c, cudaMemsetAsync(raw, 0, raw_pitch * std::max<int64_t>(m_bim, 1), c->stream));
  if (m_bim)
    SG_CUDA(c, cudaMemcpy2DAsync(raw, raw_pitch, bed + 3, nb, nb, m_bim,
                                 on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                 c->stream));
  int rc = setgeno_core(c, raw, raw_pitch, n_fam, m_bim, sub_1based, n_sub, pheno_mask, min_maf,
                        max_missing, vr_markers, n_vr, min_mac_vr, is_var_ratio, is_diag_one);
  cudaStreamSynchronize(c->stream);
  dev_free(c, raw);
  return rc;
}

extern "C" int sg_setgeno(sg_ctx* c, const uint8_t* bed, uint64_t bed_len, int64_t n_fam,
                          int64_t m_bim, const int32_t* sub_1based, int64_t n_sub,
                          const uint8_t* pheno_mask, float min_maf, float max_missing,
                          const int32_t* vr, int64_t n_vr, float min_mac_vr, int is_var_ratio,
                          int is_diag_one) {
  return setgeno_common(c, bed, false, bed_len, n_fam, m_bim, sub_1based, n_sub, pheno_mask, min_maf,
                        max_missing, vr, n_vr, min_mac_vr, is_var_ratio, is_diag_one);
}

extern "C" int sg_setgeno_device(sg_ctx* c, const uint8_t* bed_dev, uint64_t bed_len, int64_t n_fam,
                                 int64_t m_bim, const int32_t* sub_1based, int64_t n_sub,
                                 const uint8_t* pheno_mask, float min_maf, float max_missing,
                                 const int32_t* vr, int64_t n_vr, float min_mac_vr, int is_var_ratio,
                                 int is_diag_one) {
  return setgeno_common(c, bed_dev, true, bed_len, n_fam, m_bim, sub_1based, n_sub, pheno_mask,
                        min_maf, max_missing, vr, n_vr, min_mac_vr, is_var_ratio, is_diag_one);
}

static int64_t count_lines(const char* path, bool* ok) {
  std::ifstream f(path);
  if (!f.is_open()) {
    *ok = false;
    return 0;
  }
  *ok = true;
  int64_t n = 0;
  std::string s;
  while (std::getline(f, s)) ++n;
  return n;
}

extern "C" int sg_setgeno_files(sg_ctx* c, const char* bed_path, const char* bim_path,
                                const char* fam_path, const int32_t* sub_1based, int64_t n_sub,
                                const uint8_t* pheno_mask, float min_maf, float max_missing,
                                const int32_t* vr, int64_t n_vr, float min_mac_vr, int is_var_ratio,
                                int is_diag_one) {
  if (!c || !bed_path || !bim_path || !fam_path) return SG_ERR_INVALID;
  bool ok1, ok2;
  const int64_t n_fam = count_lines(fam_path, &ok1);
  const int64_t m_bim = count_lines(bim_path, &ok2);
  if (!ok1 || !ok2) return set_err(c, SG_ERR_IO, "cannot open %s", ok1 ? bim_path : fam_path);
  std::ifstream f(bed_path, std::ios::binary);
  if (!f.is_open()) return set_err(c, SG_ERR_IO, "cannot open %s", bed_path);
  std::vector<uint8_t> bytes((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  return sg_setgeno(c, bytes.data(), bytes.size(), n_fam, m_bim, sub_1based, n_sub, pheno_mask,
                    min_maf, max_missing, vr, n_vr, min_mac_vr, is_var_ratio, is_diag_one);
}

#define NEED_GENO(c) \
  do { if (!(c)) return SG_ERR_INVALID; if (!(c)->have_geno) return set_err((c), SG_ERR_STATE, "setgeno has not run"); } while (0)
#define NEED_GRM(c) \
  do { NEED_GENO(c); if (!(c)->have_grm) return set_err((c), SG_ERR_STATE, "sg_grm_build has not run"); } while (0)
// the engine's operator: the resident K, or (subset-exact engine) the genotype matrix
#define NEED_OPERATOR(c)                                                                               \
  do {                                                                                                 \
    NEED_GENO(c);                                                                                      \
    if (!(c)->have_grm && !(exact_mode((c)->mv_mode) && (c)->d_G))                                      \
      return set_err((c), SG_ERR_STATE, "sg_grm_build has not run (or select SG_MV_SUBSET_EXACT)");    \
  } while (0)

extern "C" int sg_geno_dims(sg_ctx* c, int64_t* n, int64_t* m_total, int64_t* m_qc, int64_t* m_vr) {
  NEED_GENO(c);
  if (n) *n = c->nn;
  if (m_total) *m_total = c->m_bim;
  if (m_qc) *m_qc = c->m_qc;
  if (m_vr) *m_vr = c->m_vr;
  return SG_OK;
}
extern "C" int sg_get_allele_freq(sg_ctx* c, float* out) {
  NEED_GENO(c);
  std::copy(c->freq.begin(), c->freq.end(), out);
  return SG_OK;
}
extern "C" int sg_get_invstd(sg_ctx* c, float* out) {
  NEED_GENO(c);
  std::copy(c->invstd.begin(), c->invstd.end(), out);
  return SG_OK;
}
extern "C" int sg_get_mac(sg_ctx* c, int32_t* out) {
  NEED_GENO(c);
  std::copy(c->mac.begin(), c->mac.end(), out);
  return SG_OK;
}
extern "C" int sg_get_qc_marker_mask(sg_ctx* c, uint8_t* out) {
  NEED_GENO(c);
  std::copy(c->qc_mask.begin(), c->qc_mask.end(), out);
  return SG_OK;
}
extern "C" int sg_get_vr_markers(sg_ctx* c, float* freq, int32_t* mac, int32_t* bim_index) {
  NEED_GENO(c);
  if (freq) std::copy(c->vr_freq.begin(), c->vr_freq.end(), freq);
  if (mac) std::copy(c->vr_mac.begin(), c->vr_mac.end(), mac);
  if (bim_index) std::copy(c->vr_index.begin(), c->vr_index.end(), bim_index);
  return SG_OK;
}
extern "C" int sg_get_packed_geno(sg_ctx* c, uint8_t* out) {
  NEED_GENO(c);
  const int64_t nb = (c->nn + 3) / 4;
  if (c->m_qc)
    SG_CUDA(c, cudaMemcpy2D(out, nb, c->d_packed, c->pitch, nb, c->m_qc, cudaMemcpyDeviceToHost));
  return SG_OK;
}

static int onesnp(sg_ctx* c, const uint8_t* packed, const float* lut, int64_t m, int64_t marker,
                  int32_t* g, float* z) {
  NEED_GENO(c);
  if (marker < 0 || marker >= m) return set_err(c, SG_ERR_INVALID, "marker %lld out of range", (long long)marker);
  int32_t* dg = nullptr;
  float* dz = nullptr;
  SG_TRY(dev_alloc_t(c, &dg, (size_t)c->nn));
  SG_TRY(dev_alloc_t(c, &dz, (size_t)c->nn));
  launch_unpack_marker(packed + marker * c->pitch, c->nn, lut + 4 * marker, dg, dz, c->stream);
  SG_LAUNCHED(c, 1);
  if (g) SG_CUDA(c, cudaMemcpyAsync(g, dg, c->nn * 4, cudaMemcpyDeviceToHost, c->stream));
  if (z) SG_CUDA(c, cudaMemcpyAsync(z, dz, c->nn * 4, cudaMemcpyDeviceToHost, c->stream));
  SG_TRY(sync(c));
  dev_free(c, dg);
  dev_free(c, dz);
  return SG_OK;
}
extern "C" int sg_get_onesnp_geno(sg_ctx* c, int64_t marker, int32_t* out) {
  NEED_GENO(c);
  return onesnp(c, c->d_packed, c->d_lut, c->m_qc, marker, out, nullptr);
}
extern "C" int sg_get_onesnp_geno_vr(sg_ctx* c, int64_t marker, int32_t* out) {
  NEED_GENO(c);
  return onesnp(c, c->d_packed_vr, c->d_lut_vr, c->m_vr, marker, out, nullptr);
}
extern "C" int sg_get_onesnp_stdgeno(sg_ctx* c, int64_t marker, float* out) {
  NEED_GENO(c);
  return onesnp(c, c->d_packed, c->d_lut, c->m_qc, marker, nullptr, out);
}

// ------------------------------------------------------------------ GRM build
extern "C" int sg_grm_build(sg_ctx* c, int precision) {
  NEED_GENO(c);
  if (precision != SG_GRM_FP32_SIMT && precision != SG_GRM_BF16_TC && precision != SG_GRM_BF16X3_TC)
    return set_err(c, SG_ERR_INVALID, "unknown GRM precision %d", precision);
  if (precision != SG_GRM_FP32_SIMT && !tc_available())
    return set_err(c, SG_ERR_INVALID, "tcgen05 SYRK needs an sm_103a device");
  if (c->m_qc == 0) return set_err(c, SG_ERR_STATE, "no marker passed QC");
  dev_free_t(c, c->d_K);
  dev_free_t(c, c->d_Klo);
  c->k_split = false;
  dev_free(c, c->d_Kb);
  c->d_Kb = nullptr;
  engine_free(c);
  loco_free(c);
  c->have_grm = false;
  const int64_t np = round_up(c->nn, kRowTile);
  const int64_t mp = round_up(c->m_qc, kMarkerTile);
  c->np = np;
  SG_TRY(dev_alloc_t(c, &c->d_K, (size_t)(np * np)));
  const float scale = 1.0f / (float)c->m_qc;
  if (precision == SG_GRM_FP32_SIMT) {
    float* Z = nullptr;
    SG_TRY(dev_alloc_t(c, &Z, (size_t)(np * mp)));
    SG_CUDA(c, cudaEventRecord(c->tev[0], c->stream));
    launch_zbuild_f32(c->d_packed, c->pitch, c->d_lut, c->m_qc, c->nn, np, mp, Z, c->stream);
    SG_CUDA(c, cudaEventRecord(c->tev[1], c->stream));
    launch_gemm_nt_f32(Z, mp, Z, mp, c->d_K, np, np, np, mp, scale, 2, c->stream);
    SG_LAUNCHED(c, 2);
    SG_CUDA(c, cudaEventRecord(c->tev[2], c->stream));
    SG_TRY(sync(c));
    c->t_build[3] = ev_ms(c->tev[0], c->tev[1]);
    c->t_build[4] = ev_ms(c->tev[1], c->tev[2]);
    dev_free(c, Z);
  } else {
    void* Zh = nullptr;
    void* Zl = nullptr;
    SG_TRY(dev_alloc(c, &Zh, (size_t)(np * mp * 2)));
    if (precision == SG_GRM_BF16X3_TC) SG_TRY(dev_alloc(c, &Zl, (size_t)(np * mp * 2)));
    SG_CUDA(c, cudaEventRecord(c->tev[0], c->stream));
    launch_zbuild_bf16(c->d_packed, c->pitch, c->d_lut, c->m_qc, c->nn, np, mp, Zh, Zl, c->stream);
    SG_LAUNCHED(c, 1);
    SG_CUDA(c, cudaEventRecord(c->tev[1], c->stream));
    cudaError_t e = tc_syrk_bf16(Zh, Zl, np, mp, c->d_K, scale, c->stream);
    cudaEventRecord(c->tev[2], c->stream);
    if (e != cudaSuccess) return set_err(c, SG_ERR_CUDA, "tcgen05 SYRK: %s", cudaGetErrorString(e));
    SG_LAUNCHED(c, 1);
    SG_TRY(sync(c));
    c->t_build[3] = ev_ms(c->tev[0], c->tev[1]);
    c->t_build[4] = ev_ms(c->tev[1], c->tev[2]);
    dev_free(c, Zh);
    dev_free(c, Zl);
  }
  c->have_grm = true;
  return SG_OK;
}

// Split K = Khi + Klo in place for the split-TF32 engine, or recombine it (exactly) for the others.
static int ensure_k_split(sg_ctx* c, bool want) {
  if (!c->have_grm || want == c->k_split) return SG_OK;
  const int64_t n2 = c->np * c->np;
  if (want) {
    SG_TRY(dev_alloc_t(c, &c->d_Klo, (size_t)n2));
    launch_split_tf32(c->d_K, c->d_K, c->d_Klo, n2, c->stream);
    SG_LAUNCHED(c, 1);
    c->k_split = true;
  } else {
    add_inplace_kernel<<<(unsigned)((n2 + 255) / 256), 256, 0, c->stream>>>(c->d_K, c->d_Klo, n2);
    SG_LAUNCHED(c, 1);
    SG_TRY(sync(c));
    dev_free_t(c, c->d_Klo);
    c->k_split = false;
  }
  return sync(c);
}

// BF16 high/low halves of K for the split-BF16 engine (built from the exact FP32 K, which stays
// resident for the other engines, the diagonal and sg_grm_get); freed when another engine is chosen.
static int ensure_k_bf16(sg_ctx* c, bool want) {
  if (!c->have_grm || want == (c->d_Kb != nullptr)) return SG_OK;
  if (!want) {
    SG_TRY(sync(c));
    dev_free(c, c->d_Kb);
    c->d_Kb = nullptr;
    return SG_OK;
  }
  const int64_t n2 = c->np * c->np;
  SG_TRY(dev_alloc(c, &c->d_Kb, (size_t)n2 * 4));
  launch_split_bf16(c->d_K, c->k_split ? c->d_Klo : nullptr, c->d_Kb,
                    static_cast<uint16_t*>(c->d_Kb) + n2, n2, c->stream);
  SG_LAUNCHED(c, 1);
  return sync(c);
}

extern "C" int sg_grm_padded_n(sg_ctx* c, int64_t* np) {
  NEED_OPERATOR(c);
  if (!np) return set_err(c, SG_ERR_INVALID, "null output");
  *np = c->np;
  return SG_OK;
}

// Allocation-free GRM.V for callers that cannot allocate (see include/saigegpu.h).
extern "C" int sg_grm_matmul_tf32x3_noalloc(sg_ctx* c, const float* P_dev, int64_t ncols, float* Y_dev,
                                            void* stream) {
  NEED_GRM(c);
  if (!P_dev || !Y_dev) return set_err(c, SG_ERR_INVALID, "null device pointer");
  // the scratch address is looked up per device, for the device that is current
  SG_CUDA(c, cudaSetDevice(c->device));
  if (!c->k_split)
    return set_err(c, SG_ERR_STATE, "select SG_MV_TF32X3_TC first (the split GRM is not resident)");
  if (ncols <= 0 || ncols % 32 != 0)
    return set_err(c, SG_ERR_INVALID, "ncols = %lld must be a positive multiple of 32", (long long)ncols);
  if (ncols * c->np > tc_noalloc_max_elems())
    return set_err(c, SG_ERR_INVALID, "ncols * n_p = %lld exceeds the static scratch limit of %lld entries",
                   (long long)(ncols * c->np), (long long)tc_noalloc_max_elems());
  cudaError_t e = tc_gemm_tf32x3_noalloc(c->d_K, c->d_Klo, c->np, P_dev, ncols, Y_dev,
                                         reinterpret_cast<cudaStream_t>(stream));
  c->launches += 2;
  if (e != cudaSuccess) return set_err(c, e == cudaErrorLaunchTimeout ? SG_ERR_TIMEOUT : SG_ERR_CUDA,
                                       "no-alloc GRM.V: %s", cudaGetErrorString(e));
  return SG_OK;
}

extern "C" int sg_build_timing(sg_ctx* c, double* t5) {
  if (!c || !t5) return SG_ERR_INVALID;
  for (int i = 0; i < 5; ++i) t5[i] = c->t_build[i];
  return SG_OK;
}

extern "C" int sg_grm_diag(sg_ctx* c, double* out) {
  NEED_GENO(c);
  std::copy(c->diag.begin(), c->diag.end(), out);
  return SG_OK;
}
extern "C" int sg_grm_diag_f32(sg_ctx* c, float* out) {
  NEED_GENO(c);
  std::copy(c->diag32.begin(), c->diag32.end(), out);
  return SG_OK;
}
extern "C" int sg_grm_get(sg_ctx* c, float* out) {
  NEED_GRM(c);
  SG_CUDA(c, cudaMemcpy2D(out, c->nn * 4, c->d_K, c->np * 4, c->nn * 4, c->nn, cudaMemcpyDeviceToHost));
  if (c->k_split) {
    std::vector<float> lo((size_t)(c->nn * c->nn));
    SG_CUDA(c, cudaMemcpy2D(lo.data(), c->nn * 4, c->d_Klo, c->np * 4, c->nn * 4, c->nn, cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < lo.size(); ++i) out[i] += lo[i];
  }
  return SG_OK;
}

// ------------------------------------------------------------------ engine
static cudaError_t h2d(sg_ctx* c, void* dst, const void* src, size_t bytes, cudaStream_t s) {
  c->eng.io_h2d += bytes;
  return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s);
}
static cudaError_t d2h(sg_ctx* c, void* dst, const void* src, size_t bytes, cudaStream_t s) {
  c->eng.io_d2h += bytes;
  return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s);
}

static void engine_free(sg_ctx* c) {
  Engine& e = c->eng;
  cudaStreamSynchronize(c->side);
  for (auto& x : c->setup) cudaStreamSynchronize(x);  // a weight upload may still read a staging buffer
  cudaStreamSynchronize(c->wts);
  for (double* h : e.h_wslot)
    if (h) cudaFreeHost(h);
  for (cudaEvent_t ev : e.ev_slot)
    if (ev) cudaEventDestroy(ev);
  e.h_wslot.clear();
  e.ev_slot.clear();
  e.slot_rec.clear();
  e.slot_wait.clear();
  dev_free_t(c, e.X); dev_free_t(c, e.R); dev_free_t(c, e.Z); dev_free_t(c, e.P);
  dev_free_t(c, e.B); dev_free_t(c, e.part); dev_free_t(c, e.winv); dev_free_t(c, e.minv);
  dev_free_t(c, e.Yd); dev_free_t(c, e.Pf); dev_free_t(c, e.Yf); dev_free_t(c, e.d_st);
  dev_free_t(c, e.d_ph); dev_free_t(c, e.d_cols); dev_free_t(c, e.Pflo);
  dev_free(c, e.Pb);
  e.Pb = nullptr;
  dev_free_t(c, e.d_sx); dev_free_t(c, e.d_dpart); dev_free_t(c, e.d_dcols); dev_free_t(c, e.ptab);
  dev_free_t(c, e.pcache);
  e.pcache_key.clear();
  for (auto& ss : e.sub) {
    dev_free_t(c, ss.dp); dev_free_t(c, ss.p2); dev_free_t(c, ss.lut); dev_free_t(c, ss.flips);
    dev_free_t(c, ss.dfill); dev_free_t(c, ss.bits); dev_free_t(c, ss.diag);
    dev_free_t(c, ss.qc); dev_free_t(c, ss.flag); dev_free_t(c, ss.mb); dev_free_t(c, ss.d_counts);
    if (ss.h_counts) cudaFreeHost(ss.h_counts);
    if (ss.h_mb) cudaFreeHost(ss.h_mb);
    if (ss.h_rec) cudaFreeHost(ss.h_rec);
    if (ss.ev_prep) cudaEventDestroy(ss.ev_prep);
  }
  e.sub.clear();
  e.max_w = 0;
  dev_free_t(c, e.d_slots);
  dev_free(c, e.Vb);
  e.Vb = nullptr;
  dev_free_t(c, e.Tm);
  dev_free(c, e.Tb);
  e.Tb = nullptr;
  dev_free_t(c, e.Um);
  dev_free_t(c, e.spart);
  dev_free_t(c, e.smax);
  dev_free_t(c, e.sscale);
  for (auto& p : e.sdiag_part) dev_free_t(c, p);

  e.dots_cap_sx = e.dots_cap_part = e.dots_cap_cols = 0;
  for (auto& dp : e.dots) {
    if (dp.ev) cudaEventSynchronize(dp.ev);
    if (dp.h_part) cudaFreeHost(dp.h_part);
    if (dp.ev) cudaEventDestroy(dp.ev);
  }
  e.dots.clear();
  if (e.inflight) cudaStreamSynchronize(c->stream);
  e.inflight = false;
  e.pending_release.clear();
  if (e.h_pin) cudaFreeHost(e.h_pin);
  e.h_pin = nullptr;
  if (e.h_gcols) cudaFreeHost(e.h_gcols);
  e.h_gcols = nullptr;
  for (auto& p : e.d_wstage) dev_free_t(c, p);
  dev_free_t(c, e.d_wstage2);
  for (void** hp : {reinterpret_cast<void**>(&e.h_sst), reinterpret_cast<void**>(&e.h_scol),
                    reinterpret_cast<void**>(&e.h_acols), reinterpret_cast<void**>(&e.h_ptab)}) {
    if (*hp) cudaFreeHost(*hp);
    *hp = nullptr;
  }
  dev_free_t(c, e.d_sst);
  dev_free_t(c, e.d_scol);
  e.n_sst = 0;
  if (!e.slab_blocks.empty()) cudaStreamSynchronize(c->up);
  for (void* blk : e.slab_blocks) cudaFreeHost(blk);
  e.slab_blocks.clear();
  for (void* blk : e.slab_dblocks) dev_free(c, blk);
  e.slab_dblocks.clear();
  e.slab_free.clear();
  e.up_wait = false;
  dev_free_t(c, e.d_gcols);
  e.cap_cols = e.cap_ph = 0;
  e.np = 0;
  e.finished.clear();
  dev_free_t(c, c->d_lu);
  dev_free_t(c, c->d_lv);
  dev_free_t(c, c->d_lp);
  e.hi_col = 0;
  e.n_active = 0;
  e.queue.clear();
  e.reqs.clear();
  e.deps.clear();
  e.h_st.clear();
  e.col_req.clear();
  e.ph_set.clear();
}

// Drop every queued and in-flight request (the blocking drop-ins own the engine); results are
// copied out at retirement from here on.
static int apply_releases(sg_ctx* c);
static void slab_put(Engine& e, Req& r);
static bool slab_get(sg_ctx* c, Req& r);

static int engine_clear(sg_ctx* c) {
  Engine& e = c->eng;
  e.hold = false;
  if (e.cap_cols == 0) return SG_OK;
  if (e.inflight) {  // an abandoned asynchronous step: let it drain, drop its results
    e.inflight = false;
    SG_TRY(sync(c));
  }
  SG_TRY(apply_releases(c));
  bool any = false;
  for (int64_t col = 0; col < (int64_t)e.col_req.size(); ++col) {
    if (e.col_req[col] < 0) continue;
    any = true;
    e.col_req[col] = -1;
    e.h_st[col] = ColState{};
    e.h_st[col].kind = -1;
    SG_CUDA(c, cudaMemsetAsync(e.Pf + col * e.np, 0, e.np * 4, c->stream));
  }
  if (any)
    SG_CUDA(c, cudaMemcpyAsync(e.d_st, e.h_st.data(), e.cap_cols * sizeof(ColState), cudaMemcpyHostToDevice, c->stream));
  e.hi_col = 0;
  e.n_active = 0;
  e.queue.clear();
  for (auto& kv : e.reqs) slab_put(e, kv.second);
  e.reqs.clear();
  e.deps.clear();
  return sync(c);
}

static int engine_reserve(sg_ctx* c, int64_t max_columns, int64_t max_phenos) {
  NEED_OPERATOR(c);
  Engine& e = c->eng;
  max_columns = round_up(std::max<int64_t>(max_columns, 32), 32);
  if (max_columns > 96) max_columns = round_up(max_columns, 128);
  if (max_columns > 320) max_columns = round_up(max_columns, 256);
  max_phenos = std::max<int64_t>(max_phenos, 1);
  if (max_columns > 65535)  // one grid row per column in the vector kernels
    return set_err(c, SG_ERR_INVALID, "at most 65535 engine columns (asked for %lld)", (long long)max_columns);
  if (e.cap_cols >= max_columns && e.cap_ph >= max_phenos && e.np == c->np) return SG_OK;
  for (auto& kv : e.reqs)
    if (kv.second.state == 1) return set_err(c, SG_ERR_STATE, "engine busy: cannot grow while columns run");
  max_columns = std::max(max_columns, e.np == c->np ? e.cap_cols : 0);
  max_phenos = std::max(max_phenos, e.np == c->np ? e.cap_ph : 0);
  std::vector<PhenoState> old_ph = e.h_ph;
  std::vector<char> old_set = e.ph_set;
  engine_free(c);
  const int64_t np = c->np;
  e.np = np;
  e.nblk = pcg_nblk(np);
  e.stage_cols = std::min<int64_t>(max_columns, 256);
  const size_t V = (size_t)(max_columns * np);
  SG_TRY(dev_alloc_t(c, &e.X, V)); SG_TRY(dev_alloc_t(c, &e.R, V));
  SG_TRY(dev_alloc_t(c, &e.Z, V)); SG_TRY(dev_alloc_t(c, &e.P, V));
  SG_TRY(dev_alloc_t(c, &e.Pf, V)); SG_TRY(dev_alloc_t(c, &e.Yf, V));
  SG_TRY(dev_alloc_t(c, &e.B, (size_t)(e.stage_cols * np)));
  SG_TRY(dev_alloc_t(c, &e.part, (size_t)(max_columns * e.nblk * 2)));
  SG_TRY(dev_alloc_t(c, &e.ptab, (size_t)(e.stage_cols * 36)));  // probe tables | RHS pointers and rows
  SG_TRY(dev_alloc_t(c, &e.winv, (size_t)(max_phenos * np)));
  SG_TRY(dev_alloc_t(c, &e.minv, (size_t)(max_phenos * np)));
  SG_TRY(dev_alloc_t(c, &e.d_st, (size_t)max_columns));
  SG_TRY(dev_alloc_t(c, &e.d_ph, (size_t)max_phenos));
  SG_TRY(dev_alloc_t(c, &e.d_cols, (size_t)max_columns));
  SG_CUDA(c, cudaMemsetAsync(e.Pf, 0, V * 4, c->stream));
  SG_CUDA(c, cudaMemsetAsync(e.P, 0, V * 8, c->stream));
  SG_CUDA(c, cudaMemsetAsync(e.winv, 0, (size_t)(max_phenos * np) * 8, c->stream));
  SG_CUDA(c, cudaMemsetAsync(e.minv, 0, (size_t)(max_phenos * np) * 8, c->stream));
  e.cap_cols = max_columns;
  e.cap_ph = max_phenos;
  for (auto& ev : e.ev)
    if (!ev) SG_CUDA(c, cudaEventCreate(&ev));
  for (auto& ev : e.ev_prev)
    if (!ev) SG_CUDA(c, cudaEventCreate(&ev));
  if (!e.ev_adm) SG_CUDA(c, cudaEventCreate(&e.ev_adm));
  if (!e.ev_up) SG_CUDA(c, cudaEventCreateWithFlags(&e.ev_up, cudaEventDisableTiming));
  e.have_prev = false;
  SG_CUDA(c, cudaHostAlloc(reinterpret_cast<void**>(&e.h_pin), max_columns * sizeof(ColState), cudaHostAllocDefault));
  SG_CUDA(c, cudaHostAlloc(reinterpret_cast<void**>(&e.h_gcols), max_columns * sizeof(int32_t), cudaHostAllocDefault));
  SG_CUDA(c, cudaHostAlloc(reinterpret_cast<void**>(&e.h_sst), max_columns * sizeof(ColState), cudaHostAllocDefault));
  SG_CUDA(c, cudaHostAlloc(reinterpret_cast<void**>(&e.h_scol), max_columns * sizeof(int32_t), cudaHostAllocDefault));
  SG_CUDA(c, cudaHostAlloc(reinterpret_cast<void**>(&e.h_acols), e.stage_cols * sizeof(int32_t), cudaHostAllocDefault));
  SG_CUDA(c, cudaHostAlloc(reinterpret_cast<void**>(&e.h_ptab), e.stage_cols * 36, cudaHostAllocDefault));
  SG_TRY(dev_alloc_t(c, &e.d_sst, (size_t)max_columns));
  e.stage_idx.assign(max_columns, -1);
  e.slab_pending.clear();
  SG_TRY(dev_alloc_t(c, &e.d_scol, (size_t)max_columns));
  for (auto& p : e.d_wstage) SG_TRY(dev_alloc_t(c, &p, (size_t)(2 * np)));
  SG_TRY(dev_alloc_t(c, &e.d_wstage2, (size_t)(2 * np)));
  SG_TRY(dev_alloc_t(c, &e.d_gcols, (size_t)max_columns));
  e.h_st.assign(max_columns, ColState{});
  for (auto& s : e.h_st) { s.kind = -1; s.active = 0; }
  SG_CUDA(c, cudaMemcpyAsync(e.d_st, e.h_st.data(), max_columns * sizeof(ColState), cudaMemcpyHostToDevice, c->stream));
  e.col_req.assign(max_columns, -1);
  e.h_ph.assign(max_phenos, PhenoState{0.0, 0.0});
  e.ph_set.assign(max_phenos, 0);
  e.sub.assign(max_phenos, Engine::SlotSub{});
  // per-slot records that calls made without the driver's lock read: sized here, never resized
  // while the engine runs
  e.dots.assign(max_phenos, Engine::DotsPending{});
  e.h_wslot.assign(max_phenos, nullptr);
  e.ev_slot.assign(max_phenos, nullptr);
  e.slot_rec.assign(max_phenos, 0);
  e.slot_wait.assign(max_phenos, 0);
  SG_TRY(dev_alloc_t(c, &e.d_slots, (size_t)max_phenos));
  SG_CUDA(c, cudaMemsetAsync(e.d_slots, 0, max_phenos * sizeof(SubsetSlot), c->stream));
  e.hi_col = 0;
  e.n_active = 0;
  e.queue.clear();
  e.reqs.clear();
  e.deps.clear();
  SG_TRY(sync(c));
  (void)old_ph; (void)old_set;
  return SG_OK;
}

extern "C" int sg_engine_reserve(sg_ctx* c, int64_t max_columns, int64_t max_phenos) {
  return engine_reserve(c, max_columns, max_phenos);
}

// Subset-exact engine: the state of slot ``slot``'s sample subset, rebuilt only when its mask
// changes.  The subset's per-marker counts, fill, QC, frequency and 1/sd come from the same kernel
// setgeno uses (genoClass::setGenoObj over the subset, FIT.cpp:376-385, 436-495, 916-921), run on
// the cohort's codes of every .bim marker with the subset as the phenotype mask; the host turns them
// into d' = 1/sd'^2 (GRM markers), 2p', the fill-changed markers and the diagonal table.  dmask: the
// mask bytes already on the device (set-up stream), or nullptr for every sample.
// First half of a slot's subset set-up, on the set-up stream: the subset's QC records (the kernel
// setgeno uses, run with the subset as the phenotype mask), then d', 2p', the diagonal table, the
// fill-change list and the two counts the host needs, copied to pinned memory; ev_prep marks the
// end.  Nothing here waits for the device.
static int subset_prepare(sg_ctx* c, int64_t slot, const uint8_t* mask) {
  Engine& e = c->eng;
  Engine::SlotSub& ss = e.sub[slot];
  const int64_t nn = c->nn, np = e.np, mg = c->mg, m = c->m_bim;
  const int64_t nwords = (nn + 15) / 16;
  std::vector<uint32_t> maskbits(nwords + 1, 0u);
  int64_t ns = 0;
  for (int64_t i = 0; i < nn; ++i)
    if (!mask || mask[i]) {
      maskbits[i / 16] |= 1u << (2 * (i % 16));
      ++ns;
    }
  if (ns == 0) return set_err(c, SG_ERR_INVALID, "phenotype slot %lld: empty sample subset", (long long)slot);
  // the slot's buffers (kept; the fill-change list has room for every marker)
  if (!ss.qc) SG_TRY(dev_alloc_t(c, &ss.qc, (size_t)std::max<int64_t>(m, 1)));
  if (!ss.flag) SG_TRY(dev_alloc_t(c, &ss.flag, (size_t)mg));
  if (!ss.mb) SG_TRY(dev_alloc_t(c, &ss.mb, (size_t)(nwords + 1)));
  if (!ss.d_counts) SG_TRY(dev_alloc_t(c, &ss.d_counts, (size_t)2));
  if (!ss.h_counts) SG_CUDA(c, cudaHostAlloc(reinterpret_cast<void**>(&ss.h_counts), 2 * sizeof(int64_t),
                                             cudaHostAllocDefault));
  if (!ss.ev_prep) SG_CUDA(c, cudaEventCreateWithFlags(&ss.ev_prep, cudaEventDisableTiming));
  if (!ss.dp) SG_TRY(dev_alloc_t(c, &ss.dp, (size_t)mg));
  if (!ss.p2) SG_TRY(dev_alloc_t(c, &ss.p2, (size_t)mg));
  if (!ss.lut) SG_TRY(dev_alloc_t(c, &ss.lut, (size_t)(4 * mg)));
  if (!ss.diag) SG_TRY(dev_alloc_t(c, &ss.diag, (size_t)np));
  if (!ss.flips) SG_TRY(dev_alloc_t(c, &ss.flips, (size_t)std::max<int64_t>(m, 1)));
  if (!ss.dfill) SG_TRY(dev_alloc_t(c, &ss.dfill, (size_t)std::max<int64_t>(m, 1)));
  if (!ss.h_mb) SG_CUDA(c, cudaHostAlloc(reinterpret_cast<void**>(&ss.h_mb), (nwords + 1) * sizeof(uint32_t),
                                         cudaHostAllocDefault));
  if (ss.prep) SG_CUDA(c, cudaEventSynchronize(ss.ev_prep));  // an earlier prepare still owns the buffers
  // (the last prepare's copy out of h_mb has completed: a set-up waited for its ev_prep)
  std::memcpy(ss.h_mb, maskbits.data(), maskbits.size() * 4);
  const int q = (int)(slot % kSetupStreams);
  cudaStream_t st = c->setup[q];
  SG_CUDA(c, cudaMemcpyAsync(ss.mb, ss.h_mb, maskbits.size() * 4, cudaMemcpyHostToDevice, st));
  launch_marker_qc(c->d_codes, c->pitch, m, nn, ss.mb, ns, c->qc_min_maf, c->qc_max_missing, c->d_vrflag_all,
                   c->qc_min_mac_vr, c->qc_max_mac_vr, c->qc_is_var_ratio, ss.qc, st);
  // d' = 1/sd'^2, 2p' and the diagonal table per marker, the fill-changed markers in marker order,
  // on the device (setGenoObj's per-marker values over the subset, FIT.cpp:436-495, 152-159)
  launch_subset_derive(ss.qc, c->d_fill_all, m, mg, c->sub_loco_lo, c->sub_loco_hi, ss.dp, ss.p2, ss.lut, ss.flag,
                       ss.flips, ss.dfill, ss.d_counts, st);
  SG_CUDA(c, cudaMemcpyAsync(ss.h_counts, ss.d_counts, 2 * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  SG_CUDA(c, cudaEventRecord(ss.ev_prep, st));
  // the diagonal needs only the tables: it follows here, after the counts the host waits for
  // (the slot's weights, later on this stream, read it)
  if (!e.sdiag_part[q]) SG_TRY(dev_alloc_t(c, &e.sdiag_part[q], (size_t)subset_diag_scratch(m, np)));
  launch_subset_diag(c->d_codes, c->pitch, ss.lut, m, nn, np, e.sdiag_part[q], ss.diag, st);
  SG_LAUNCHED(c, 5);
  ss.valid = false;
  ss.prep = true;
  ss.prep_all = mask == nullptr;
  if (mask) ss.prep_mask.assign(mask, mask + nn);
  else ss.prep_mask.clear();
  ss.prep_ns = ns;
  ss.prep_lo = c->sub_loco_lo;
  ss.prep_hi = c->sub_loco_hi;
  return SG_OK;
}

static bool same_mask(bool all, const std::vector<uint8_t>& kept, const uint8_t* mask, int64_t nn) {
  return (!mask && all) || (mask && !all && std::memcmp(kept.data(), mask, nn) == 0);
}
// the slot's built / prepared subset state is the one for this mask and the context's LOCO range
static bool slot_built(const sg_ctx* c, const Engine::SlotSub& ss, const uint8_t* mask) {
  return ss.valid && ss.ex_lo == c->sub_loco_lo && ss.ex_hi == c->sub_loco_hi && same_mask(ss.all, ss.mask, mask, c->nn);
}
static bool slot_prepared(const sg_ctx* c, const Engine::SlotSub& ss, const uint8_t* mask) {
  return ss.prep && ss.prep_lo == c->sub_loco_lo && ss.prep_hi == c->sub_loco_hi &&
         same_mask(ss.prep_all, ss.prep_mask, mask, c->nn);
}

// Subset-exact engine: the state of slot ``slot``'s sample subset, rebuilt only when its mask
// changes.  The subset's per-marker counts, fill, QC, frequency and 1/sd come from the same kernel
// setgeno uses (genoClass::setGenoObj over the subset, FIT.cpp:376-385, 436-495, 916-921), run on
// the cohort's codes of every .bim marker with the subset as the phenotype mask; the device turns
// them into d' = 1/sd'^2 (GRM markers), 2p', the fill-changed markers and the diagonal table.
// dmask: the mask bytes already on the device (set-up stream), or nullptr for every sample.  The
// first half runs here unless sg_engine_prepare_subset launched it for this mask already.
static int subset_setup(sg_ctx* c, int64_t slot, const uint8_t* mask, const uint8_t* dmask) {
  Engine& e = c->eng;
  Engine::SlotSub& ss = e.sub[slot];
  const int64_t nn = c->nn, np = e.np, m = c->m_bim;
  if (slot_built(c, ss, mask)) return SG_OK;
  if (!slot_prepared(c, ss, mask)) SG_TRY(subset_prepare(c, slot, mask));
  SG_CUDA(c, cudaEventSynchronize(ss.ev_prep));
  ss.prep = false;
  const int64_t nflip = ss.h_counts[0], mprime = ss.h_counts[1], ns = ss.prep_ns;
  if (mprime == 0) return set_err(c, SG_ERR_STATE, "phenotype slot %lld: no marker passes QC in its subset", (long long)slot);
  const int W = (int)((nflip + 31) / 32);
  if ((int64_t)W * np > ss.bits_cap) {
    // with room to spare (cudaFree waits for the whole device, steps included): at least 64 words
    // (2,048 fill changes) a sample, then half again what this subset needs
    const int64_t words = std::max<int64_t>(64, ((int64_t)W * 3 / 2 + 31) / 32 * 32);
    dev_free_t(c, ss.bits);
    SG_TRY(dev_alloc_t(c, &ss.bits, (size_t)(words * np)));
    ss.bits_cap = words * np;
  }
  cudaStream_t st = c->setup[slot % kSetupStreams];
  launch_subset_bitmap(c->d_codes, c->pitch, ss.flips, (int)nflip, W, dmask, nn, np, ss.bits, st);
  SG_LAUNCHED(c, W > 0 ? 1 : 0);
  ss.dev.dprime = ss.dp;
  ss.dev.p2 = ss.p2;
  ss.dev.flips = ss.flips;
  ss.dev.dfill = ss.dfill;
  ss.dev.bits = ss.bits;
  ss.dev.nflip = (int32_t)nflip;
  ss.dev.W = W;
  ss.dev.inv_m = 1.0 / (double)mprime;
  ss.dev.ns = (double)ns;
  // through the slot's pinned record, so the call does not wait for the stream (the slot's last
  // record copy has completed: set_pheno waited for the slot's event)
  if (!ss.h_rec) SG_CUDA(c, cudaHostAlloc(reinterpret_cast<void**>(&ss.h_rec), sizeof(SubsetSlot), cudaHostAllocDefault));
  *ss.h_rec = ss.dev;
  SG_CUDA(c, cudaMemcpyAsync(e.d_slots + slot, ss.h_rec, sizeof(SubsetSlot), cudaMemcpyHostToDevice, st));
  ss.m_prime = (double)mprime;
  ss.all = ss.prep_all;
  ss.ex_lo = ss.prep_lo;
  ss.ex_hi = ss.prep_hi;
  ss.mask.swap(ss.prep_mask);
  ss.prep_mask.clear();
  ss.valid = true;
  // over every slot's device record, kept ones included: a forgotten slot's columns may still run
  e.max_w = 0;
  for (const auto& x : e.sub) e.max_w = std::max(e.max_w, (int)x.dev.W);
  return SG_OK;
}

extern "C" int sg_engine_prepare_subset(sg_ctx* c, int64_t slot, const uint8_t* mask) {
  NEED_OPERATOR(c);
  Engine& e = c->eng;
  if (!exact_mode(c->mv_mode)) return SG_OK;  // the other engines keep no subset state
  if (e.cap_ph == 0) SG_TRY(engine_reserve(c, 128, std::max<int64_t>(slot + 1, 1)));
  if (slot < 0 || slot >= e.cap_ph) return set_err(c, SG_ERR_INVALID, "phenotype slot %lld out of range", (long long)slot);
  for (auto& kv : e.reqs)
    if (kv.second.state == 1 && kv.second.slot == slot)
      return set_err(c, SG_ERR_STATE, "phenotype slot %lld has columns in flight", (long long)slot);
  Engine::SlotSub& ss = e.sub[slot];
  if (slot_built(c, ss, mask) || slot_prepared(c, ss, mask)) return SG_OK;
  return subset_prepare(c, slot, mask);
}

// Reads only the slot's event (set by the prepare this thread made), so the caller may wait here
// without serialising with other threads' engine calls.
extern "C" int sg_engine_subset_wait(sg_ctx* c, int64_t slot) {
  if (!c) return SG_ERR_INVALID;
  Engine& e = c->eng;
  if (slot < 0 || slot >= (int64_t)e.sub.size()) return SG_OK;
  const Engine::SlotSub& ss = e.sub[slot];
  if (ss.prep && ss.ev_prep) (void)cudaEventSynchronize(ss.ev_prep);
  return SG_OK;
}

// The variance-ratio markers of a slot's subset, as setgeno over the subset selects them (the random
// draw's markers with MAC >= min over the subset, or the categorical ranges; FIT.cpp:497-547): their
// .bim indices in marker order and MAC over the subset.  From the QC records of the slot's last set-up.
extern "C" int sg_engine_subset_vr_markers(sg_ctx* c, int64_t slot, int32_t* bim_index, int32_t* mac, int64_t cap,
                                           int64_t* n) {
  NEED_OPERATOR(c);
  Engine& e = c->eng;
  if (!exact_mode(c->mv_mode)) return set_err(c, SG_ERR_STATE, "select a subset-exact engine first");
  if (slot < 0 || slot >= (int64_t)e.sub.size() || !e.sub[slot].valid || !e.sub[slot].qc)
    return set_err(c, SG_ERR_STATE, "phenotype slot %lld has no subset set up", (long long)slot);
  const int64_t m = c->m_bim;
  std::vector<MarkerQC> qc(m);
  if (m) SG_CUDA(c, cudaMemcpyAsync(qc.data(), e.sub[slot].qc, m * sizeof(MarkerQC), cudaMemcpyDeviceToHost, c->side));
  SG_TRY(sync_side(c));
  int64_t k = 0;
  for (int64_t i = 0; i < m; ++i) {
    if (!qc[i].pass_vr) continue;
    if (k < cap) {
      if (bim_index) bim_index[k] = (int32_t)i;
      if (mac) mac[k] = qc[i].mac;
    }
    ++k;
  }
  if (n) *n = k;
  return SG_OK;
}

// Genotypes (0/1/2) of .bim marker ``marker`` for every cohort sample, missing calls taking the fill
// of the slot's subset (Get_OneSNP_Geno over the subset's setgeno, FIT.cpp:346-357, 447).
extern "C" int sg_engine_subset_geno(sg_ctx* c, int64_t slot, int64_t marker, int32_t* out) {
  NEED_OPERATOR(c);
  Engine& e = c->eng;
  if (!out) return set_err(c, SG_ERR_INVALID, "null output");
  if (!exact_mode(c->mv_mode)) return set_err(c, SG_ERR_STATE, "select a subset-exact engine first");
  if (slot < 0 || slot >= (int64_t)e.sub.size() || !e.sub[slot].valid || !e.sub[slot].qc)
    return set_err(c, SG_ERR_STATE, "phenotype slot %lld has no subset set up", (long long)slot);
  if (marker < 0 || marker >= c->m_bim) return set_err(c, SG_ERR_INVALID, "marker %lld out of range", (long long)marker);
  std::vector<uint8_t> row((size_t)c->pitch);
  MarkerQC q{};
  SG_CUDA(c, cudaMemcpyAsync(row.data(), c->d_codes + marker * c->pitch, c->pitch, cudaMemcpyDeviceToHost, c->side));
  SG_CUDA(c, cudaMemcpyAsync(&q, e.sub[slot].qc + marker, sizeof(MarkerQC), cudaMemcpyDeviceToHost, c->side));
  SG_TRY(sync_side(c));
  for (int64_t i = 0; i < c->nn; ++i) {
    const unsigned f = (row[i >> 2] >> (2 * (i & 3))) & 3u;
    out[i] = f == 1u ? q.fill : 2 - (int)((f & 1u) + (f >> 1));
  }
  return SG_OK;
}

extern "C" int sg_engine_forget_subsets(sg_ctx* c) {
  NEED_OPERATOR(c);
  for (auto& ss : c->eng.sub) {
    ss.valid = false;
    if (ss.prep) cudaEventSynchronize(ss.ev_prep);
    ss.prep = false;
  }
  return SG_OK;
}

// A slot's weights: 1/W and the Jacobi preconditioner from getDiagOfSigma in FP64
// (FIT.cpp:2322-2365); with a chromosome left out, getDiagOfSigma_LOCO (FIT.cpp:2370-2392): diag
// minus the chromosome's sum z^2, over M - M_j.
extern "C" int sg_engine_set_pheno(sg_ctx* c, int64_t slot, const double* w, const double* tau,
                                   const uint8_t* mask) {
  NEED_OPERATOR(c);
  Engine& e = c->eng;
  if (e.cap_ph == 0) SG_TRY(engine_reserve(c, 128, std::max<int64_t>(slot + 1, 1)));
  if (slot < 0 || slot >= e.cap_ph) return set_err(c, SG_ERR_INVALID, "phenotype slot %lld out of range", (long long)slot);
  if (!w || !tau) return set_err(c, SG_ERR_INVALID, "null w/tau");
  if (!all_finite(tau, 2)) return set_err(c, SG_ERR_NUMERIC, "tau is not finite");
  for (int64_t i = 0; i < c->nn; ++i)
    if ((!mask || mask[i]) && !(std::isfinite(w[i]) && w[i] > 0.0))
      return set_err(c, SG_ERR_NUMERIC, "W[%lld] = %g is not a positive finite weight", (long long)i, w[i]);
  for (auto& kv : e.reqs)
    if (kv.second.state == 1 && kv.second.slot == slot)
      return set_err(c, SG_ERR_STATE, "phenotype slot %lld has columns in flight", (long long)slot);
  // W (and the sample mask) go up through the slot's pinned staging; 1/W and the Jacobi
  // preconditioner 1/diag(Sigma) are formed on the device from the resident FP64 diagonal
  if ((int64_t)e.ev_slot.size() < e.cap_ph) {
    e.h_wslot.resize(e.cap_ph, nullptr);
    e.ev_slot.resize(e.cap_ph, nullptr);
    e.slot_rec.resize(e.cap_ph, 0);
    e.slot_wait.resize(e.cap_ph, 0);
  }
  if (!e.ev_slot[slot]) SG_CUDA(c, cudaEventCreateWithFlags(&e.ev_slot[slot], cudaEventDisableTiming));
  // the slot's pinned staging: W (np doubles), the mask (np bytes), then its PhenoState
  const size_t ph_off = (e.np * (sizeof(double) + 1) + 15) / 16 * 16;
  if (!e.h_wslot[slot])
    SG_CUDA(c, cudaHostAlloc(reinterpret_cast<void**>(&e.h_wslot[slot]), ph_off + sizeof(PhenoState),
                             cudaHostAllocDefault));
  if (e.slot_rec[slot]) SG_CUDA(c, cudaEventSynchronize(e.ev_slot[slot]));  // its last upload (long done)
  // a slot whose subset is (re)built uploads behind its set-up on the set-up stream; a slot already
  // set up only needs new weights, on the weights stream (its set-up completed: ev_slot above)
  const bool rebuild = exact_mode(c->mv_mode) && !slot_built(c, e.sub[slot], mask);
  cudaStream_t us = rebuild ? c->setup[slot % kSetupStreams] : c->wts;
  {
    double* hw = e.h_wslot[slot];
    uint8_t* hm = reinterpret_cast<uint8_t*>(e.h_wslot[slot] + e.np);
    std::memcpy(hw, w, c->nn * sizeof(double));
    if (mask) std::memcpy(hm, mask, c->nn);
    const bool loco = c->loco && !c->is_diag_one;
    const double m = loco ? (double)(c->m_qc - c->loco_mj) : (double)c->m_qc;
    double* dw = rebuild ? e.d_wstage[slot % kSetupStreams] : e.d_wstage2;
    uint8_t* dm = reinterpret_cast<uint8_t*>(dw + e.np);
    SG_CUDA(c, h2d(c, dw, hw, c->nn * sizeof(double), us));
    if (mask) SG_CUDA(c, h2d(c, dm, hm, c->nn, us));
    const double* diag = loco ? c->d_diag_loco : c->d_diag;
    double mm = m;
    if (exact_mode(c->mv_mode)) {  // the subset's own diagonal and GRM marker count
      SG_TRY(subset_setup(c, slot, mask, mask ? dm : nullptr));
      diag = e.sub[slot].diag;
      mm = e.sub[slot].m_prime;
    }
    launch_slot_weights(e.np, c->nn, dw, mask ? dm : nullptr, diag, mm, tau[0], tau[1],
                        c->is_diag_one ? 1 : 0, e.winv + slot * e.np, e.minv + slot * e.np, us);
    SG_LAUNCHED(c, 1);
  }
  e.h_ph[slot] = PhenoState{tau[0], tau[1]};
  PhenoState* hph = reinterpret_cast<PhenoState*>(reinterpret_cast<uint8_t*>(e.h_wslot[slot]) + ph_off);
  *hph = e.h_ph[slot];
  SG_CUDA(c, h2d(c, e.d_ph + slot, hph, sizeof(PhenoState), us));
  e.ph_set[slot] = 1;
  SG_CUDA(c, cudaEventRecord(e.ev_slot[slot], us));
  e.slot_rec[slot] = e.slot_wait[slot] = 1;
  return SG_OK;
}

static int engine_submit_common(sg_ctx* c, int64_t slot, int kind, const double* B, bool probe,
                                uint64_t seed, int64_t run0, int64_t k, int maxiter, double tol,
                                int64_t* ids) {
  NEED_OPERATOR(c);
  Engine& e = c->eng;
  if (slot < 0 || slot >= e.cap_ph || !e.ph_set[slot])
    return set_err(c, SG_ERR_STATE, "phenotype slot %lld not set", (long long)slot);
  if (kind != 0 && kind != 1) return set_err(c, SG_ERR_INVALID, "kind must be 0 or 1");
  if (k < 0 || (!probe && k > 0 && !B)) return set_err(c, SG_ERR_INVALID, "bad RHS block");
  if (!probe && !all_finite(B, k * c->nn)) return set_err(c, SG_ERR_NUMERIC, "right-hand side has NaN/Inf");
  for (int64_t j = 0; j < k; ++j) {
    Req r;
    r.id = e.next_id++;
    r.slot = slot;
    r.kind = kind;
    r.maxiter = maxiter;
    r.tol = tol;
    r.probe = probe;
    r.seed = seed;
    r.run = run0 + j;
    if (!probe) {
      if (!slab_get(c, r)) return set_err(c, SG_ERR_NOMEM, "no memory for a right-hand side's slab");
      std::memcpy(r.b, B + j * c->nn, c->nn * sizeof(double));
      // up now, on the upload stream, while the step in flight runs: admission gathers on the device
      SG_CUDA(c, cudaMemcpyAsync(const_cast<double*>(r.bd), r.b, c->nn * sizeof(double), cudaMemcpyHostToDevice,
                                 c->up));
      e.io_h2d += (uint64_t)(c->nn * 8);
    }
    if (ids) ids[j] = r.id;
    e.queue.push_back(r.id);
    e.reqs.emplace(r.id, std::move(r));
  }
  if (!probe && k > 0) {
    SG_CUDA(c, cudaEventRecord(e.ev_up, c->up));
    e.up_wait = true;
  }
  return SG_OK;
}

extern "C" int sg_engine_submit(sg_ctx* c, int64_t slot, int kind, const double* B, int64_t k,
                                int maxiter, double tol, int64_t* ids) {
  return engine_submit_common(c, slot, kind, B, false, 0, 0, k, maxiter, tol, ids);
}
extern "C" int sg_engine_submit_probes(sg_ctx* c, int64_t slot, int kind, uint64_t seed, int64_t run0,
                                       int64_t k, int maxiter, double tol, int64_t* ids) {
  return engine_submit_common(c, slot, kind, nullptr, true, seed, run0, k, maxiter, tol, ids);
}

extern "C" int sg_engine_submit_chained(sg_ctx* c, int64_t slot, const int64_t* src_ids, int64_t k, int maxiter,
                                        double tol, int64_t* ids) {
  NEED_OPERATOR(c);
  Engine& e = c->eng;
  if (!e.hold) return set_err(c, SG_ERR_STATE, "chained solves need held results (sg_engine_hold_results)");
  if (slot < 0 || slot >= e.cap_ph || !e.ph_set[slot])
    return set_err(c, SG_ERR_STATE, "phenotype slot %lld not set", (long long)slot);
  if (k < 0 || (k > 0 && !src_ids)) return set_err(c, SG_ERR_INVALID, "bad source list");
  for (int64_t j = 0; j < k; ++j)
    if (!e.reqs.count(src_ids[j]))
      return set_err(c, SG_ERR_NOT_FOUND, "unknown source request %lld", (long long)src_ids[j]);
  for (int64_t j = 0; j < k; ++j) {
    Req r;
    r.id = e.next_id++;
    r.slot = slot;
    r.kind = 0;
    r.maxiter = maxiter;
    r.tol = tol;
    r.src = src_ids[j];
    // a slab for the source's result, should the source be fetched before this one is admitted
    if (!slab_get(c, r)) return set_err(c, SG_ERR_NOMEM, "no pinned host memory for a right-hand side");
    if (ids) ids[j] = r.id;
    e.deps.emplace(r.src, r.id);
    e.queue.push_back(r.id);
    e.reqs.emplace(r.id, std::move(r));
  }
  return SG_OK;
}

// Column-state updates go up in one block: stage (col, state) pairs, then flush_states copies them
// and scatters them into d_st with one launch.  The pinned staging is reused only after the stream
// has drained past the copy (wait = true, or a later synchronisation on the same stream).
static void stage_state(Engine& e, int64_t col, const ColState& st) {
  int32_t& at = e.stage_idx[col];
  if (at >= 0) {  // staged earlier in this batch (released, then admitted again): the last state wins
    e.h_sst[at] = st;
    return;
  }
  at = (int32_t)e.n_sst;
  e.h_sst[e.n_sst] = st;
  e.h_scol[e.n_sst] = (int32_t)col;
  ++e.n_sst;
}

static int flush_states(sg_ctx* c, bool wait) {
  Engine& e = c->eng;
  if (e.n_sst == 0) return SG_OK;
  const int64_t n = e.n_sst;
  e.n_sst = 0;
  for (int64_t k = 0; k < n; ++k) e.stage_idx[e.h_scol[k]] = -1;
  SG_CUDA(c, cudaMemcpyAsync(e.d_sst, e.h_sst, n * sizeof(ColState), cudaMemcpyHostToDevice, c->stream));
  SG_CUDA(c, cudaMemcpyAsync(e.d_scol, e.h_scol, n * sizeof(int32_t), cudaMemcpyHostToDevice, c->stream));
  e.io_h2d += (uint64_t)(n * (sizeof(ColState) + sizeof(int32_t)));
  launch_scatter_states(e.d_sst, e.d_scol, n, e.d_st, e.Pf, e.np, c->stream);
  SG_LAUNCHED(c, 1);
  return wait ? sync(c) : SG_OK;
}

// Slabs of nn doubles for queued right-hand sides, each a pinned host buffer and a device buffer
// (grown 32 at a time, kept until the engine is freed): a submission copies its right-hand side
// into the host slab and uploads it to the device slab on the upload stream at once; admission's
// gather kernel reads the device slab.
static bool slab_get(sg_ctx* c, Req& r) {
  Engine& e = c->eng;
  if (e.slab_free.empty()) {
    constexpr int64_t kPer = 32;
    const size_t bytes = (size_t)(kPer * c->nn) * sizeof(double);
    void* blk = nullptr;
    if (cudaHostAlloc(&blk, bytes, cudaHostAllocDefault) != cudaSuccess) return false;
    void* dblk = nullptr;
    if (dev_alloc(c, &dblk, bytes) != SG_OK) {
      cudaFreeHost(blk);
      return false;
    }
    e.slab_blocks.push_back(blk);
    e.slab_dblocks.push_back(dblk);
    for (int64_t k = 0; k < kPer; ++k)
      e.slab_free.emplace_back(static_cast<double*>(blk) + k * c->nn, static_cast<const double*>(dblk) + k * c->nn);
  }
  r.b = e.slab_free.back().first;
  r.bd = e.slab_free.back().second;
  e.slab_free.pop_back();
  return true;
}

static void slab_put(Engine& e, Req& r) {
  if (r.b) e.slab_free.emplace_back(r.b, r.bd);
  r.b = nullptr;
  r.bd = nullptr;
}

// Move queued requests into free columns, staged through e.B, and initialise them.
static void unlink_dep(Engine& e, int64_t src, int64_t dep) {
  auto range = e.deps.equal_range(src);
  for (auto it = range.first; it != range.second; ++it)
    if (it->second == dep) {
      e.deps.erase(it);
      return;
    }
}

// Before a finished request's column is released: the chained requests still queued on it get its
// result in their own right-hand-side slabs.  Before an unfinished one is cancelled: they are
// cancelled with it (their right-hand side will never exist).
static int detach_dependents(sg_ctx* c, Req& src) {
  Engine& e = c->eng;
  auto range = e.deps.equal_range(src.id);
  if (range.first == range.second) return SG_OK;
  std::vector<int64_t> ds;
  for (auto it = range.first; it != range.second; ++it) ds.push_back(it->second);
  e.deps.erase(src.id);
  bool copied = false;
  for (int64_t d : ds) {
    auto it = e.reqs.find(d);
    if (it == e.reqs.end()) continue;
    Req& r = it->second;
    if (src.state == 2 && src.col >= 0 && r.bd) {
      SG_CUDA(c, cudaMemcpyAsync(const_cast<double*>(r.bd), e.X + src.col * e.np, c->nn * 8,
                                 cudaMemcpyDeviceToDevice, c->side));
      r.src = -1;
      copied = true;
    } else {
      slab_put(e, r);
      e.reqs.erase(it);  // its queue entry is skipped at admission
    }
  }
  return copied ? sync_side(c) : SG_OK;
}

static int engine_admit(sg_ctx* c) {
  Engine& e = c->eng;
  if (e.up_wait) {  // right-hand sides uploaded since the last admission (long since, as a rule)
    SG_CUDA(c, cudaStreamWaitEvent(c->stream, e.ev_up, 0));
    e.up_wait = false;
  }

  // the previous admission's copies have run (the stream drained at the last finish / sync)
  for (int64_t id : e.slab_pending) {
    auto it = e.reqs.find(id);
    if (it != e.reqs.end()) slab_put(e, it->second);
  }
  e.slab_pending.clear();
  SG_TRY(apply_releases(c));
  bool synced_round = false;
  while (!e.queue.empty()) {
    if (synced_round) {  // a second round reuses the staging buffers and e.B: wait for the first
      SG_TRY(sync(c));
      for (int64_t id : e.slab_pending) {
        auto it = e.reqs.find(id);
        if (it != e.reqs.end()) slab_put(e, it->second);
      }
      e.slab_pending.clear();
    }
    synced_round = true;
    std::vector<int32_t> cols;
    std::vector<int64_t> admitted;
    std::vector<uint64_t> pseeds;
    std::vector<int64_t> pruns;
    std::vector<int32_t> psel;
    std::vector<const double*> rsrc;
    std::vector<int32_t> rsel;
    int64_t col = 0;
    std::vector<int64_t> later;  // chained requests whose source has not finished: stay queued, in order
    while (!e.queue.empty() && (int64_t)cols.size() < e.stage_cols) {
      while (col < e.cap_cols && e.col_req[col] != -1) ++col;
      if (col >= e.cap_cols) break;
      const int64_t id = e.queue.front();
      e.queue.pop_front();
      auto it = e.reqs.find(id);
      if (it == e.reqs.end()) continue;  // cancelled
      Req& r = it->second;
      if (r.slot < (int64_t)e.slot_wait.size() && e.slot_wait[r.slot]) {
        // the slot's weights (and subset set-up) were uploaded on the set-up stream since its last
        // admission: admit once they are there; while other columns run, leave it for a later step
        // rather than hold the step back
        if (cudaEventQuery(e.ev_slot[r.slot]) == cudaSuccess) {
          e.slot_wait[r.slot] = 0;
        } else if (e.n_active > 0 || !cols.empty()) {
          later.push_back(id);
          continue;
        } else {
          SG_CUDA(c, cudaStreamWaitEvent(c->stream, e.ev_slot[r.slot], 0));
          e.slot_wait[r.slot] = 0;
          ++e.adm_waits;
        }
      }
      const int64_t sel = (int64_t)cols.size();
      if (r.src >= 0) {
        auto is = e.reqs.find(r.src);
        if (is == e.reqs.end() || is->second.state != 2 || is->second.col < 0) {
          later.push_back(id);
          continue;
        }
        rsrc.push_back(e.X + is->second.col * e.np);  // the source's result, still in its column
        rsel.push_back((int32_t)sel);
        unlink_dep(e, r.src, id);
        r.src = -1;
      } else if (r.probe) {
        pseeds.push_back(r.seed);
        pruns.push_back(r.run);
        psel.push_back((int32_t)sel);
      } else {
        rsrc.push_back(r.bd);  // the device slab, uploaded at submission
        rsel.push_back((int32_t)sel);
      }
      ColState s{};
      s.pheno = (int32_t)r.slot;
      s.kind = r.kind;
      s.maxiter = r.maxiter;
      s.tol = r.tol;
      stage_state(e, col, s);
      // the device decides at init whether the column iterates; until the step's states come back
      // the host counts it as active (the GRM.V then includes it; a column that converged at init
      // is skipped by the vector kernels and retired when the step finishes)
      e.h_st[col] = s;
      e.h_st[col].active = 1;
      e.col_req[col] = id;
      r.col = col;
      r.state = 1;
      cols.push_back((int32_t)col);
      admitted.push_back(id);
      e.hi_col = std::max(e.hi_col, col + 1);
      ++col;
    }
    e.queue.insert(e.queue.begin(), later.begin(), later.end());
    if (cols.empty()) break;
    SG_TRY(flush_states(c, false));  // the round's closing synchronisation frees the staging
    if (!rsrc.empty()) {
      // explicit right-hand sides: pointer and row tables staged behind the probe tables
      const size_t kr = rsrc.size();
      unsigned char* hb = e.h_ptab + e.stage_cols * 24;
      std::memcpy(hb, rsrc.data(), kr * sizeof(void*));
      std::memcpy(hb + kr * sizeof(void*), rsel.data(), kr * 4);
      unsigned char* db = reinterpret_cast<unsigned char*>(e.ptab) + e.stage_cols * 24;
      SG_CUDA(c, h2d(c, db, hb, kr * (sizeof(void*) + 4), c->stream));
      launch_gather_rhs(reinterpret_cast<const double* const*>(db), reinterpret_cast<const int32_t*>(db + kr * sizeof(void*)),
                        (int64_t)kr, c->nn, e.np, e.B, c->stream);
      SG_LAUNCHED(c, 1);
    }
    if (!psel.empty()) {
      // one launch for every probe of this admission round; its index table (uint64 seeds |
      // int64 runs | int32 rows, at most stage_cols entries) is staged in pinned memory, then e.ptab
      const size_t kp = psel.size();
      uint64_t* h_seeds = reinterpret_cast<uint64_t*>(e.h_ptab);
      int64_t* h_runs = reinterpret_cast<int64_t*>(h_seeds + kp);
      int32_t* h_sel = reinterpret_cast<int32_t*>(h_runs + kp);
      std::memcpy(h_seeds, pseeds.data(), kp * 8);
      std::memcpy(h_runs, pruns.data(), kp * 8);
      std::memcpy(h_sel, psel.data(), kp * 4);
      SG_CUDA(c, h2d(c, e.ptab, e.h_ptab, kp * 20, c->stream));
      uint64_t* d_seeds = reinterpret_cast<uint64_t*>(e.ptab);
      int64_t* d_runs = reinterpret_cast<int64_t*>(d_seeds + kp);
      int32_t* d_sel = reinterpret_cast<int32_t*>(d_runs + kp);
      launch_probe_fill_multi(e.np, c->nn, d_seeds, d_runs, d_sel, (int64_t)kp, e.B, c->stream);
      c->launches += 1;
    }
    std::memcpy(e.h_acols, cols.data(), cols.size() * 4);
    SG_CUDA(c, h2d(c, e.d_cols, e.h_acols, cols.size() * 4, c->stream));
    launch_pcg_init(e.np, e.cap_cols, e.d_cols, (int64_t)cols.size(), e.d_st, e.d_ph, e.minv, e.B,
                    e.X, e.R, e.Z, e.P, e.Pf, e.part, e.nblk, c->stream);
    SG_LAUNCHED(c, 2);
    // for the FP64 plain engine the product columns read P: stage b there too
    if (c->mv_mode == SG_MV_FP64_PLAIN) {
      for (size_t k = 0; k < cols.size(); ++k) {
        if (e.h_st[cols[k]].kind == 1)
          SG_CUDA(c, cudaMemcpyAsync(e.P + (int64_t)cols[k] * e.np, e.B + (int64_t)k * e.np, e.np * 8,
                                     cudaMemcpyDeviceToDevice, c->stream));
      }
    }
    // the staging buffers and slabs are reused only after the stream has drained past init
    e.slab_pending.insert(e.slab_pending.end(), admitted.begin(), admitted.end());
    e.n_active += (int64_t)cols.size();
    if ((int64_t)cols.size() < e.stage_cols) break;
  }
  return flush_states(c, false);  // releases with no admission round after them
}

static int loco_correct(sg_ctx* c, int64_t ncols, bool yf);
static int engine_gemm_full(sg_ctx* c, int64_t ncols, bool* used_yf, int64_t* launched);

// GRM product of the step: Y = K P for the columns in [0, ncols); *launched = the columns the
// tensor-core kernel computed (the active ones, compacted and padded, in the split-BF16 engine).
static int engine_gemm(sg_ctx* c, int64_t ncols, bool* used_yf, int64_t* launched) {
  SG_TRY(engine_gemm_full(c, ncols, used_yf, launched));
  if (c->loco) SG_TRY(loco_correct(c, ncols, *used_yf));
  return SG_OK;
}

static int engine_gemm_full(sg_ctx* c, int64_t ncols, bool* used_yf, int64_t* launched) {
  Engine& e = c->eng;
  *used_yf = true;
  *launched = ncols;
  if (c->mv_mode == SG_MV_FP64_PLAIN) {
    *used_yf = false;
    if (!e.Yd) SG_TRY(dev_alloc_t(c, &e.Yd, (size_t)(e.cap_cols * e.np)));
    for (int64_t col = 0; col < ncols; ++col) {
      if (!e.h_st[col].active) continue;
      launch_gemv_f64(c->d_K, e.np, e.np, e.P + col * e.np, e.Yd + col * e.np, c->stream);
      c->launches += 1;
    }
    return SG_OK;
  }
  if (c->mv_mode == SG_MV_BF16X3_TC) {
    if (!c->d_Kb) SG_TRY(ensure_k_bf16(c, true));
    const size_t half = (size_t)(e.cap_cols * e.np);
    if (!e.Pb) SG_TRY(dev_alloc(c, &e.Pb, half * 4));
    // only the columns still iterating are multiplied: their P is gathered into a compact block
    // (padded with zero columns to the tile width) and the epilogue scatters Y back by column
    const int64_t nact = e.nact;  // built by step_launch
    if (nact == 0) {
      *launched = 0;
      return SG_OK;
    }
    const int64_t npad = tc_grmv_padded_cols(round_up(nact, 16), e.cap_cols, e.np, kTilesSplitBF16, c->num_sms);
    for (int64_t j = nact; j < npad; ++j) e.h_gcols[j] = -1;
    SG_CUDA(c, cudaMemcpyAsync(e.d_gcols, e.h_gcols, npad * 4, cudaMemcpyHostToDevice, c->stream));
    uint16_t* ph = static_cast<uint16_t*>(e.Pb);
    launch_split_bf16_gather(e.Pf, e.np, e.d_gcols, npad, ph, ph + half, c->stream);
    c->launches += 1;
    *launched = npad;
    const uint16_t* kh = static_cast<const uint16_t*>(c->d_Kb);
    cudaError_t err = tc_gemm_bf16x3(kh, kh + c->np * c->np, e.np, ph, ph + half, npad, e.Yf, c->stream, false,
                                     e.d_gcols);
    if (err != cudaSuccess) return set_err(c, SG_ERR_CUDA, "tcgen05 GRM.V: %s", cudaGetErrorString(err));
    c->launches += 1;
    return SG_OK;
  }
  if (exact_mode(c->mv_mode)) {
    // K_S P per column's own sample subset, through the genotype matrix (k_subset.cu)
    const int64_t nact = e.nact;
    if (nact == 0) {
      *launched = 0;
      return SG_OK;
    }
    const int64_t np = e.np, mg = c->mg;
    const int64_t npad = tc_grmv_padded_cols(round_up(nact, 32), e.cap_cols, np, kTilesSplitB, c->num_sms);
    for (int64_t j = nact; j < npad; ++j) e.h_gcols[j] = -1;
    SG_CUDA(c, cudaMemcpyAsync(e.d_gcols, e.h_gcols, npad * 4, cudaMemcpyHostToDevice, c->stream));
    const size_t cap = (size_t)e.cap_cols;
    if (!e.Vb) SG_TRY(dev_alloc(c, &e.Vb, cap * np * 4));
    if (!e.Tm) SG_TRY(dev_alloc_t(c, &e.Tm, cap * mg));
    if (!e.Tb) SG_TRY(dev_alloc(c, &e.Tb, cap * mg * 4));
    if (!e.Um) SG_TRY(dev_alloc_t(c, &e.Um, cap * np));
    if (!e.spart) SG_TRY(dev_alloc_t(c, &e.spart, cap * (size_t)std::max(subset_nblk(np), subset_nblk(mg))));
    uint16_t* vh = static_cast<uint16_t*>(e.Vb);
    uint16_t* vl = vh + cap * np;
    uint16_t* th = static_cast<uint16_t*>(e.Tb);
    uint16_t* tl = th + cap * mg;
    const uint16_t* Gmm = static_cast<const uint16_t*>(c->d_G);
    const uint16_t* Gsm = Gmm + mg * np;
    if (c->mv_mode == SG_MV_SUBSET_EXACT_F8) {
      // FP16 high halves (2 bytes) then E4M3 low halves (1 byte) in the same buffers
      const size_t nb = (size_t)std::max(subset_nblk(np), subset_nblk(mg));
      if (!e.smax) SG_TRY(dev_alloc_t(c, &e.smax, cap * nb));
      if (!e.sscale) SG_TRY(dev_alloc_t(c, &e.sscale, 2 * cap));
      uint8_t* vl8 = reinterpret_cast<uint8_t*>(vh + cap * np);
      uint8_t* tl8 = reinterpret_cast<uint8_t*>(th + cap * mg);
      const uint8_t* Gmm8 = reinterpret_cast<const uint8_t*>(Gmm + 2 * mg * np);
      const uint8_t* Gsm8 = Gmm8 + mg * np;
      launch_subset_prepare_f8(e.Pf, np, e.d_gcols, npad, e.d_st, e.d_slots, e.winv, e.spart, e.smax, vh, vl8,
                               e.sscale, c->stream);
      c->launches += 2;
      cudaError_t err = tc_gemm_splitb8(Gmm, Gmm8, mg, np, vh, vl8, npad, e.Tm, mg, c->stream, false, 0);
      if (err != cudaSuccess) return set_err(c, SG_ERR_CUDA, "tcgen05 genotype GEMM (G'V): %s", cudaGetErrorString(err));
      launch_subset_scale_f8(vh, vl8, np, c->nn, e.d_gcols, npad, e.d_st, e.d_slots, e.max_w, e.Tm, mg, th, tl8,
                             e.spart, e.smax, e.sscale, (int64_t)cap, c->stream);
      c->launches += e.max_w > 0 ? 4 : 3;
      err = tc_gemm_splitb8(Gsm, Gsm8, np, mg, th, tl8, npad, e.Um, np, c->stream, false, 1);
      if (err != cudaSuccess) return set_err(c, SG_ERR_CUDA, "tcgen05 genotype GEMM (G T'): %s", cudaGetErrorString(err));
      launch_subset_finalize_f8(e.Um, np, c->nn, e.d_gcols, npad, e.d_st, e.d_slots, th, tl8, mg, e.sscale + cap,
                                e.spart, e.winv, e.Yf, c->stream);
      c->launches += 2;
      SG_LAUNCHED(c, 0);
      *launched = npad;
      return SG_OK;
    }
    launch_subset_prepare(e.Pf, np, e.d_gcols, npad, e.d_st, e.d_slots, e.winv, e.spart, vh, vl, c->stream);
    c->launches += 2;
    cudaError_t err = tc_gemm_splitb(Gmm, mg, np, vh, vl, npad, e.Tm, mg, c->stream, false, 0);
    if (err != cudaSuccess) return set_err(c, SG_ERR_CUDA, "tcgen05 genotype GEMM (G'V): %s", cudaGetErrorString(err));
    launch_subset_scale(vh, vl, np, c->nn, e.d_gcols, npad, e.d_st, e.d_slots, e.max_w, e.Tm, mg, th, tl, e.spart,
                        c->stream);
    c->launches += e.max_w > 0 ? 3 : 2;
    err = tc_gemm_splitb(Gsm, np, mg, th, tl, npad, e.Um, np, c->stream, false, 1);
    if (err != cudaSuccess) return set_err(c, SG_ERR_CUDA, "tcgen05 genotype GEMM (G T'): %s", cudaGetErrorString(err));
    launch_subset_finalize(e.Um, np, c->nn, e.d_gcols, npad, e.d_st, e.d_slots, th, tl, mg, e.spart, e.winv, e.Yf,
                           c->stream);
    c->launches += 2;
    SG_LAUNCHED(c, 0);
    *launched = npad;
    return SG_OK;
  }
  if (c->mv_mode == SG_MV_TF32_TC || c->mv_mode == SG_MV_TF32X3_TC) {
    const bool split = c->mv_mode == SG_MV_TF32X3_TC;
    if (split) {
      if (!c->k_split) SG_TRY(ensure_k_split(c, true));
      if (!e.Pflo) SG_TRY(dev_alloc_t(c, &e.Pflo, (size_t)(e.cap_cols * e.np)));
      launch_split_tf32(e.Pf, e.Pf, e.Pflo, ncols * e.np, c->stream);
      c->launches += 1;
    }
    cudaError_t err = tc_gemm_tf32(c->d_K, split ? c->d_Klo : nullptr, e.np, e.Pf,
                                   split ? e.Pflo : nullptr, ncols, e.Yf, c->stream, false);
    if (err != cudaSuccess) return set_err(c, SG_ERR_CUDA, "tcgen05 GRM.V: %s", cudaGetErrorString(err));
    c->launches += 1;
    return SG_OK;
  }
  launch_gemm_nt_f32(c->d_K, e.np, e.Pf, e.np, e.Yf, e.np, e.np, ncols, e.np, 1.0f, 1, c->stream);
  c->launches += 1;
  return SG_OK;
}

// One engine step over columns [0, hi_col): GRM product + the FP64 PCG vector work.
static int release_col(sg_ctx* c, int64_t col);

// Columns the GRM.V of one step covers: [0, hi_col) padded to the kernel's column tile (the
// padding columns are free or finished, their P rows are zero).
static bool tc_mode(int mode) {
  return mode == SG_MV_TF32_TC || mode == SG_MV_TF32X3_TC || mode == SG_MV_BF16X3_TC || exact_mode(mode);
}
// engines that gather the step's active columns into a compact block themselves
static bool compact_mode(int mode) { return mode == SG_MV_BF16X3_TC || exact_mode(mode); }

static int64_t engine_gemm_cols(const sg_ctx* c) {
  const Engine& e = c->eng;
  const int64_t ncols = round_up(e.hi_col, 32);
  if (!tc_mode(c->mv_mode)) return ncols;
  return tc_grmv_padded_cols(ncols, e.cap_cols, e.np, c->mv_mode == SG_MV_TF32_TC ? kTilesPlain : kTilesSplitTF32,
                             c->num_sms);
}

// First half of a step over columns [0, hi_col): GRM product + the FP64 PCG vector work, the
// step's timing events and an asynchronous read-back of the column states into pinned memory.
// Nothing here waits for the device.
static int step_launch(sg_ctx* c) {
  Engine& e = c->eng;
  // the step's active columns (host view: admitted columns count as active until their state comes
  // back); the GRM.V compaction and the vector kernels work on this list only
  e.nact = 0;
  for (int64_t col = 0; col < e.hi_col; ++col)
    if (e.h_st[col].active) e.h_gcols[e.nact++] = (int32_t)col;
  // the split-BF16 engine compacts the active columns itself; the others cover [0, hi_col) padded
  const int64_t ncols = compact_mode(c->mv_mode) ? round_up(e.hi_col, 32) : engine_gemm_cols(c);
  int64_t occupied = 0;
  for (int64_t col = 0; col < e.hi_col; ++col) occupied += e.h_st[col].active ? 1 : 0;
  bool yf = true;
  int64_t launched = ncols;
  std::swap(e.ev, e.ev_prev);  // keep the last step's events for the idle time before this one
  SG_CUDA(c, cudaEventRecord(e.ev[0], c->stream));
  SG_TRY(engine_gemm(c, ncols, &yf, &launched));
  SG_CUDA(c, cudaEventRecord(e.ev[1], c->stream));
  const float* Yf = yf ? e.Yf : nullptr;
  const double* Yd = yf ? nullptr : e.Yd;
  if (!compact_mode(c->mv_mode) && e.nact > 0)  // the compacting engines uploaded the list already
    SG_CUDA(c, cudaMemcpyAsync(e.d_gcols, e.h_gcols, e.nact * 4, cudaMemcpyHostToDevice, c->stream));
  launch_pcg_sigma_dot(e.np, e.nact, e.d_st, e.d_ph, e.winv, e.minv, e.P, Yf, Yd, e.part, e.nblk, e.d_gcols,
                       c->stream);
  launch_pcg_alpha(e.nact, e.d_st, e.part, e.nblk, e.d_gcols, c->stream);
  launch_pcg_update(e.np, e.nact, e.d_st, e.d_ph, e.winv, e.minv, e.X, e.R, e.Z, e.P, Yf, Yd,
                    e.part, e.nblk, e.d_gcols, c->stream);
  launch_pcg_beta(e.nact, e.d_st, e.part, e.nblk, e.d_gcols, c->stream);
  launch_pcg_dir(e.np, e.nact, e.d_st, e.Z, e.P, e.Pf, e.d_gcols, c->stream);
  SG_LAUNCHED(c, 5);
  SG_CUDA(c, cudaEventRecord(e.ev[2], c->stream));
  SG_CUDA(c, d2h(c, e.h_pin, e.d_st, e.hi_col * sizeof(ColState), c->stream));
  e.inflight = true;
  e.inflight_ncols = launched;
  e.inflight_occupied = occupied;
  e.inflight_hi = e.hi_col;
  return SG_OK;
}

// Second half: wait for the step, account its time, retire the columns that finished (result
// held in X[col], or copied out and the column freed).
static int step_finish(sg_ctx* c, int64_t* n_finished) {
  Engine& e = c->eng;
  e.inflight = false;
  SG_TRY(sync(c));
  const auto th0 = std::chrono::steady_clock::now();
  if (tc_mode(c->mv_mode)) {
    const cudaError_t err = tc_check_error(c->stream);
    if (err != cudaSuccess) return set_err(c, SG_ERR_CUDA, "tcgen05 GRM.V: %s", cudaGetErrorString(err));
  }
  const int64_t ncols = e.inflight_ncols, occupied = e.inflight_occupied, hi = e.inflight_hi;
  {
    float ms_gemm = 0.f, ms_step = 0.f, ms_idle = 0.f;
    cudaEventElapsedTime(&ms_gemm, e.ev[0], e.ev[1]);
    cudaEventElapsedTime(&ms_step, e.ev[0], e.ev[2]);
    if (e.have_prev && cudaEventElapsedTime(&ms_idle, e.ev_prev[2], e.ev[0]) == cudaSuccess && ms_idle > 0.f)
      e.t_idle_ms += ms_idle;
    float ms_adm = 0.f;
    if (e.adm_recorded && cudaEventElapsedTime(&ms_adm, e.ev_adm, e.ev[0]) == cudaSuccess && ms_adm > 0.f)
      e.t_admit_ms += ms_adm;
    e.adm_recorded = false;
    const bool had_prev = e.have_prev;
    e.have_prev = true;
    if ((int64_t)e.trace.size() < kStepTrace * kTraceFields) {
      const double rec[kTraceFields] = {(double)(c->mv_mode == SG_MV_FP64_PLAIN ? occupied : ncols),
                                        (double)occupied, ms_gemm, ms_step, had_prev ? (double)ms_idle : -1.0,
                                        e.inflight_gap_ms, e.inflight_launch_ms, (double)e.inflight_waits};
      e.trace.insert(e.trace.end(), rec, rec + kTraceFields);
    }
    e.t_gemm_ms += ms_gemm;
    e.t_step_ms += ms_step;
    const int64_t launched_cols = c->mv_mode == SG_MV_FP64_PLAIN ? occupied : ncols;
    e.gemm_launches += c->mv_mode == SG_MV_FP64_PLAIN ? (double)occupied : 1.0;
    e.gemm_cols += (double)launched_cols;
    e.useful_cols += (double)occupied;
    e.gemm_flops += 2.0 * (double)c->nn * (double)c->nn * (double)launched_cols;
  }
  e.steps += 1;
  e.grm_passes += 1;
  // columns released while the step ran keep their host state (free); the rest take the device's
  for (int64_t col = 0; col < hi; ++col)
    if (e.col_req[col] >= 0) e.h_st[col] = e.h_pin[col];
  int64_t fin = 0;
  for (int64_t col = 0; col < hi; ++col) {
    const int64_t id = e.col_req[col];
    if (id < 0) continue;
    ColState& s = e.h_st[col];
    if (s.kind == -2) continue;  // finished earlier, result held in X[col]
    if (s.active || s.iter > 0 || s.kind == 1) e.col_iters += 1;  // not the ones that converged at init
    if (s.active) continue;
    auto it = e.reqs.find(id);
    if (it != e.reqs.end()) {
      Req& r = it->second;
      r.iters = s.kind == 1 ? 1 : s.iter;
      r.state = 2;
      r.col = col;
      e.finished.push_back(id);
      if (!e.hold) {  // copy the result out now and free the column
        r.x.resize(c->nn);
        SG_CUDA(c, d2h(c, r.x.data(), e.X + col * e.np, c->nn * 8, c->stream));
        r.col = -1;
      }
    }
    e.n_active -= 1;
    e.retired += 1;
    ++fin;
    if (it != e.reqs.end() && it->second.col == col) {
      s.kind = -2;  // held: result stays in X[col]
      s.active = 0;
      s.just_done = 0;
      stage_state(e, col, s);
    } else {
      SG_TRY(release_col(c, col));
    }
  }
  while (e.hi_col > 0 && e.col_req[e.hi_col - 1] == -1) --e.hi_col;
  SG_TRY(flush_states(c, false));
  SG_TRY(sync(c));
  *n_finished += fin;
  e.t_fin_end = std::chrono::steady_clock::now();
  e.have_fin_end = true;
  e.t_finish_host_ms += std::chrono::duration<double, std::milli>(e.t_fin_end - th0).count();
  return SG_OK;
}

static int engine_step(sg_ctx* c, int64_t* n_finished) {
  SG_TRY(step_launch(c));
  return step_finish(c, n_finished);
}

// Columns admitted with r'r <= tol retire without a step (iter = 0, x = 0).
static int engine_retire_immediate(sg_ctx* c, int64_t* n_finished) {
  Engine& e = c->eng;
  if (e.hi_col == 0) return SG_OK;
  SG_CUDA(c, d2h(c, e.h_st.data(), e.d_st, e.hi_col * sizeof(ColState), c->stream));
  SG_TRY(sync(c));
  for (int64_t col = 0; col < e.hi_col; ++col) {
    const int64_t id = e.col_req[col];
    if (id < 0) continue;
    ColState& s = e.h_st[col];
    if (s.kind != 0 || s.active || !s.just_done) continue;
    auto it = e.reqs.find(id);
    if (it != e.reqs.end()) {
      it->second.iters = 0;
      it->second.state = 2;
      it->second.col = e.hold ? col : -1;  // X[col] was zeroed at admission
      if (!e.hold) it->second.x.assign(c->nn, 0.0);
      e.finished.push_back(id);
    }
    e.n_active -= 1;
    e.retired += 1;
    *n_finished += 1;
    if (e.hold && it != e.reqs.end()) {
      s.kind = -2;
      s.just_done = 0;
      stage_state(e, col, s);
    } else {
      SG_TRY(release_col(c, col));
    }
  }
  while (e.hi_col > 0 && e.col_req[e.hi_col - 1] == -1) --e.hi_col;
  SG_TRY(flush_states(c, false));
  return sync(c);
}

extern "C" int sg_engine_run(sg_ctx* c, int64_t max_steps, int64_t* n_finished) {
  NEED_OPERATOR(c);
  Engine& e = c->eng;
  if (e.cap_cols == 0) return set_err(c, SG_ERR_STATE, "engine not reserved");
  int64_t fin = 0;
  if (e.inflight) {
    SG_TRY(step_finish(c, &fin));
    if (fin > 0 || max_steps <= 0) {
      if (n_finished) *n_finished = fin;
      return SG_OK;
    }
  }
  for (int64_t s = 0; s < max_steps; ++s) {
    SG_TRY(engine_admit(c));
    SG_TRY(engine_retire_immediate(c, &fin));
    if (fin > 0) break;
    if (e.n_active == 0) {
      if (!e.queue.empty())
        return set_err(c, SG_ERR_STATE,
                       "engine full: %lld queued columns wait for columns that hold unconsumed results",
                       (long long)e.queue.size());
      break;
    }
    SG_TRY(engine_step(c, &fin));
    if (fin > 0) break;
  }
  if (n_finished) *n_finished = fin;
  return SG_OK;
}

// Asynchronous stepping: sg_engine_launch starts one step and returns at once; sg_engine_finish
// waits for it and retires its finished columns.  Between the two the caller may fetch held
// results, run probe reductions, upload weights of idle slots and submit work (it joins the next
// launch); those calls use the side and set-up streams and never wait for the step.
extern "C" int sg_engine_launch(sg_ctx* c, int64_t* n_finished, int* launched) {
  NEED_OPERATOR(c);
  Engine& e = c->eng;
  if (e.cap_cols == 0) return set_err(c, SG_ERR_STATE, "engine not reserved");
  if (e.inflight) return set_err(c, SG_ERR_STATE, "a step is in flight: finish it first");
  int64_t fin = 0;
  if (launched) *launched = 0;
  const auto tl0 = std::chrono::steady_clock::now();
  const double gap_ms =
      e.have_fin_end ? std::chrono::duration<double, std::milli>(tl0 - e.t_fin_end).count() : -1.0;
  e.adm_waits = 0;
  SG_CUDA(c, cudaEventRecord(e.ev_adm, c->stream));
  e.adm_recorded = true;
  SG_TRY(engine_admit(c));
  // no read-back of the fresh columns here: ones that converged at init retire when this step
  // finishes, so the launch path never waits for the device
  if (n_finished) *n_finished = fin;
  if (e.n_active == 0) {
    if (!e.queue.empty() && fin == 0)
      return set_err(c, SG_ERR_STATE,
                     "engine full: %lld queued columns wait for columns that hold unconsumed results",
                     (long long)e.queue.size());
    return SG_OK;
  }
  SG_TRY(step_launch(c));
  e.inflight_gap_ms = gap_ms;
  e.inflight_launch_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tl0).count();
  e.inflight_waits = e.adm_waits;
  if (launched) *launched = 1;
  return SG_OK;
}

extern "C" int sg_engine_finish(sg_ctx* c, int64_t* n_finished) {
  if (!c) return SG_ERR_INVALID;
  int64_t fin = 0;
  if (c->eng.inflight) SG_TRY(step_finish(c, &fin));
  if (n_finished) *n_finished = fin;
  return SG_OK;
}

// Block until the step in flight has run on the device, without finishing it.  It reads only the
// in-flight flag (written by launch and finish) and records no error, so the thread that launches
// and finishes steps may wait here while other threads make engine calls; a device error surfaces
// in the sg_engine_finish that follows.
extern "C" int sg_engine_wait(sg_ctx* c) {
  if (!c) return SG_ERR_INVALID;
  if (c->eng.inflight) (void)cudaStreamSynchronize(c->stream);
  return SG_OK;
}

// Free a column (running or holding a result) for the next admission.  The host bookkeeping is
// immediate; the device-side reset (state, zero P) waits for the next launch, so a release never
// queues behind a step in flight.
static int release_col(sg_ctx* c, int64_t col) {
  Engine& e = c->eng;
  ColState s{};
  s.kind = -1;
  s.active = 0;
  e.h_st[col] = s;
  e.col_req[col] = -1;
  e.pending_release.push_back(col);
  while (e.hi_col > 0 && e.col_req[e.hi_col - 1] == -1) --e.hi_col;
  return SG_OK;
}

static int apply_releases(sg_ctx* c) {
  Engine& e = c->eng;
  if (e.pending_release.empty()) return SG_OK;
  ColState s{};
  s.kind = -1;
  s.active = 0;
  for (int64_t col : e.pending_release) {
    if (e.col_req[col] != -1) continue;  // reused since: admission initialises it
    e.h_st[col] = s;
    stage_state(e, col, s);  // the scatter also zeroes the column's P; admission flushes the batch
  }
  e.pending_release.clear();
  return SG_OK;
}

extern "C" int sg_engine_fetch(sg_ctx* c, int64_t id, double* x, int32_t* iters) {
  if (!c) return SG_ERR_INVALID;
  Engine& e = c->eng;
  auto it = e.reqs.find(id);
  if (it == e.reqs.end()) return set_err(c, SG_ERR_NOT_FOUND, "unknown request %lld", (long long)id);
  Req& r = it->second;
  if (r.state != 2) return set_err(c, SG_ERR_STATE, "request %lld not finished", (long long)id);
  SG_TRY(detach_dependents(c, r));
  if (r.col >= 0) {
    if (x) SG_CUDA(c, d2h(c, x, e.X + r.col * e.np, c->nn * 8, c->side));
    SG_TRY(release_col(c, r.col));
    SG_TRY(sync_side(c));
  } else if (x) {
    std::copy(r.x.begin(), r.x.end(), x);
  }
  if (iters) *iters = r.iters;
  e.reqs.erase(it);
  return SG_OK;
}

extern "C" int sg_engine_cancel(sg_ctx* c, int64_t id) {
  if (!c) return SG_ERR_INVALID;
  Engine& e = c->eng;
  auto it = e.reqs.find(id);
  if (it == e.reqs.end()) return set_err(c, SG_ERR_NOT_FOUND, "unknown request %lld", (long long)id);
  Req& r = it->second;
  SG_TRY(detach_dependents(c, r));
  if (r.src >= 0) unlink_dep(e, r.src, r.id);
  if ((r.state == 1 || r.state == 2) && r.col >= 0) {
    if (r.state == 1) e.n_active -= 1;
    SG_TRY(release_col(c, r.col));
  }
  slab_put(e, r);
  e.reqs.erase(it);  // a queued id is skipped at admission
  return SG_OK;
}

// Hutchinson probe reductions on the device (see include/saigegpu.h).
static constexpr int kProbeCache = 64;

static int pcache_find(const Engine& e, int64_t slot, uint64_t seed, int64_t run) {
  if (slot >= (int64_t)e.pcache_key.size()) return -1;
  const auto& v = e.pcache_key[slot];
  for (size_t i = 0; i < v.size(); ++i)
    if (v[i].first == seed && v[i].second == run) return (int)i;
  return -1;
}

extern "C" int sg_engine_probe_cache_clear(sg_ctx* c, int64_t slot) {
  if (!c) return SG_ERR_INVALID;
  Engine& e = c->eng;
  if (slot < 0) {
    for (auto& v : e.pcache_key) v.clear();
  } else if (slot < (int64_t)e.pcache_key.size()) {
    e.pcache_key[slot].clear();
  }
  return SG_OK;
}

extern "C" int sg_engine_probe_cached(sg_ctx* c, int64_t slot, uint64_t seed, int64_t run) {
  if (!c) return 0;
  return pcache_find(c->eng, slot, seed, run) >= 0 ? 1 : 0;
}

// Probe reductions in two halves: _begin checks the requests, caches K u, uploads SX and the
// column pointers and launches the reduction on the side stream with its block partials copied to
// pinned memory (nothing waits); _wait blocks until they have arrived; _end adds them up in a fixed
// order and releases the 2k results.  One reduction per slot at a time.
extern "C" int sg_engine_probe_dots_begin(sg_ctx* c, int64_t slot, const int64_t* ids_pcg, const int64_t* ids_prod,
                                          int64_t k, uint64_t seed, int64_t run0, const double* SX, int64_t p) {
  NEED_OPERATOR(c);
  Engine& e = c->eng;
  if (k <= 0 || !ids_pcg || !ids_prod || p < 0 || p > kProbeDotsMaxP || (p > 0 && !SX))
    return set_err(c, SG_ERR_INVALID, "probe_dots: bad arguments (p <= %d)", kProbeDotsMaxP);
  if (slot < 0 || slot >= e.cap_ph) return set_err(c, SG_ERR_INVALID, "bad slot");
  if ((int64_t)e.dots.size() < e.cap_ph) e.dots.resize(e.cap_ph);
  Engine::DotsPending& dp = e.dots[slot];
  if (dp.pending) return set_err(c, SG_ERR_STATE, "slot %lld has a probe reduction in flight", (long long)slot);
  if ((int64_t)e.pcache_key.size() < e.cap_ph) e.pcache_key.resize(e.cap_ph);
  if (!e.pcache) SG_TRY(dev_alloc_t(c, &e.pcache, (size_t)(e.cap_ph * kProbeCache * e.np)));
  // Su from held engine columns; Au from a held column (then cached) or from the slot's cache
  std::vector<const double*> su(k), au(k);
  for (int64_t j = 0; j < k; ++j) {
    auto it = e.reqs.find(ids_pcg[j]);
    if (it == e.reqs.end()) return set_err(c, SG_ERR_NOT_FOUND, "unknown request %lld", (long long)ids_pcg[j]);
    if (it->second.state != 2 || it->second.col < 0)
      return set_err(c, SG_ERR_STATE, "request %lld has no resident result", (long long)ids_pcg[j]);
    su[j] = e.X + it->second.col * e.np;
    if (ids_prod[j] < 0) {
      const int ci = pcache_find(e, slot, seed, run0 + j);
      if (ci < 0) return set_err(c, SG_ERR_STATE, "probe %lld of slot %lld is not cached", (long long)(run0 + j), (long long)slot);
      au[j] = e.pcache + (slot * kProbeCache + ci) * e.np;
    } else {
      auto ia = e.reqs.find(ids_prod[j]);
      if (ia == e.reqs.end()) return set_err(c, SG_ERR_NOT_FOUND, "unknown request %lld", (long long)ids_prod[j]);
      if (ia->second.state != 2 || ia->second.col < 0)
        return set_err(c, SG_ERR_STATE, "request %lld has no resident result", (long long)ids_prod[j]);
      au[j] = e.X + ia->second.col * e.np;
      auto& keys = e.pcache_key[slot];
      int ci = pcache_find(e, slot, seed, run0 + j);
      if (ci < 0 && (int)keys.size() < kProbeCache) {
        keys.emplace_back(seed, run0 + j);
        ci = (int)keys.size() - 1;
      }
      if (ci >= 0) {
        double* dst = e.pcache + (slot * kProbeCache + ci) * e.np;
        SG_CUDA(c, cudaMemcpyAsync(dst, au[j], e.np * 8, cudaMemcpyDeviceToDevice, c->side));
        au[j] = dst;
      }
    }
  }
  const int64_t nv = 2 + 2 * p;
  const int64_t nblk = e.nblk;
  const size_t need_sx = (size_t)std::max<int64_t>(p, 1) * e.np;
  const size_t need_part = (size_t)(k * nblk * nv);
  if (e.dots_cap_sx < need_sx) {
    dev_free_t(c, e.d_sx);
    SG_TRY(dev_alloc_t(c, &e.d_sx, need_sx));
    e.dots_cap_sx = need_sx;
  }
  if (e.dots_cap_part < need_part || e.dots_cap_cols < (size_t)(2 * k)) {
    dev_free_t(c, e.d_dpart);
    dev_free_t(c, e.d_dcols);
    SG_TRY(dev_alloc_t(c, &e.d_dpart, need_part));
    SG_TRY(dev_alloc_t(c, &e.d_dcols, (size_t)(2 * k) * 2));  // 2k pointers as int64 pairs
    e.dots_cap_part = need_part;
    e.dots_cap_cols = (size_t)(2 * k);
  }
  if (dp.cap < need_part) {
    if (dp.h_part) cudaFreeHost(dp.h_part);
    dp.h_part = nullptr;
    dp.cap = 0;
    SG_CUDA(c, cudaHostAlloc(reinterpret_cast<void**>(&dp.h_part), need_part * 8, cudaHostAllocDefault));
    dp.cap = need_part;
  }
  if (!dp.ev) SG_CUDA(c, cudaEventCreateWithFlags(&dp.ev, cudaEventDisableTiming));
  // the scratch above is shared by the slots; their reductions queue on the side stream in order,
  // after the slot's last weight upload (set-up stream)
  if (slot < (int64_t)e.ev_slot.size() && e.slot_rec[slot]) SG_CUDA(c, cudaStreamWaitEvent(c->side, e.ev_slot[slot], 0));
  if (p > 0) {
    SG_CUDA(c, cudaMemsetAsync(e.d_sx, 0, need_sx * 8, c->side));
    SG_CUDA(c, cudaMemcpy2DAsync(e.d_sx, e.np * 8, SX, c->nn * 8, c->nn * 8, p, cudaMemcpyHostToDevice, c->side));
    e.io_h2d += (uint64_t)(c->nn * 8 * p);
  }
  std::vector<const double*> ptrs(su);
  ptrs.insert(ptrs.end(), au.begin(), au.end());
  SG_CUDA(c, h2d(c, e.d_dcols, ptrs.data(), ptrs.size() * sizeof(void*), c->side));
  launch_probe_dots(e.np, c->nn, reinterpret_cast<const double* const*>(e.d_dcols), k,
                    e.minv + slot * e.np, seed, run0, e.d_sx, p, e.d_dpart, nblk, c->side);
  SG_LAUNCHED(c, 1);
  SG_CUDA(c, d2h(c, dp.h_part, e.d_dpart, need_part * 8, c->side));
  SG_CUDA(c, cudaEventRecord(dp.ev, c->side));
  dp.ids_pcg.assign(ids_pcg, ids_pcg + k);
  dp.ids_prod.assign(ids_prod, ids_prod + k);
  dp.k = k;
  dp.nv = nv;
  dp.nblk = nblk;
  dp.pending = true;
  return SG_OK;
}

// Reads only the slot's event (set by the _begin this thread made).
extern "C" int sg_engine_probe_dots_wait(sg_ctx* c, int64_t slot) {
  if (!c) return SG_ERR_INVALID;
  Engine& e = c->eng;
  if (slot < 0 || slot >= (int64_t)e.dots.size()) return SG_OK;
  const Engine::DotsPending& dp = e.dots[slot];
  if (dp.pending && dp.ev) (void)cudaEventSynchronize(dp.ev);
  return SG_OK;
}

extern "C" int sg_engine_probe_dots_end(sg_ctx* c, int64_t slot, double* out, int32_t* iters) {
  NEED_OPERATOR(c);
  Engine& e = c->eng;
  if (!out) return set_err(c, SG_ERR_INVALID, "probe_dots: null output");
  if (slot < 0 || slot >= (int64_t)e.dots.size() || !e.dots[slot].pending)
    return set_err(c, SG_ERR_STATE, "slot %lld has no probe reduction in flight", (long long)slot);
  Engine::DotsPending& dp = e.dots[slot];
  SG_CUDA(c, cudaEventSynchronize(dp.ev));
  dp.pending = false;
  const int64_t k = dp.k, nv = dp.nv, nblk = dp.nblk;
  for (int64_t j = 0; j < k; ++j)
    for (int64_t v = 0; v < nv; ++v) {
      double acc = 0.0;
      for (int64_t b = 0; b < nblk; ++b) acc += dp.h_part[(j * nblk + b) * nv + v];
      out[j * nv + v] = acc;
    }
  for (int64_t j = 0; j < 2 * k; ++j) {
    const int64_t id = j < k ? dp.ids_pcg[j] : dp.ids_prod[j - k];
    if (id < 0) continue;
    auto it = e.reqs.find(id);
    if (it == e.reqs.end()) continue;
    if (iters && j < k) iters[j] = it->second.iters;
    SG_TRY(detach_dependents(c, it->second));
    SG_TRY(release_col(c, it->second.col));
    e.reqs.erase(it);
  }
  // the reduction (and the K u cache copies before it) read the released columns before ev, so a
  // later admission may overwrite them; nothing else of the side stream is waited for here
  return SG_OK;
}

extern "C" int sg_engine_probe_dots(sg_ctx* c, int64_t slot, const int64_t* ids_pcg,
                                    const int64_t* ids_prod, int64_t k, uint64_t seed, int64_t run0,
                                    const double* SX, int64_t p, double* out, int32_t* iters) {
  if (!out) return set_err(c, SG_ERR_INVALID, "probe_dots: null output");
  SG_TRY(sg_engine_probe_dots_begin(c, slot, ids_pcg, ids_prod, k, seed, run0, SX, p));
  return sg_engine_probe_dots_end(c, slot, out, iters);
}

extern "C" int sg_engine_hold_results(sg_ctx* c, int hold) {
  if (!c) return SG_ERR_INVALID;
  c->eng.hold = hold != 0;
  return SG_OK;
}

extern "C" int sg_engine_poll(sg_ctx* c, int64_t* ids, int64_t max_ids, int64_t* n_out) {
  if (!c || !n_out || (max_ids > 0 && !ids)) return SG_ERR_INVALID;
  Engine& e = c->eng;
  const int64_t k = std::min<int64_t>(max_ids, (int64_t)e.finished.size());
  for (int64_t i = 0; i < k; ++i) ids[i] = e.finished[i];
  e.finished.erase(e.finished.begin(), e.finished.begin() + k);
  *n_out = k;
  return SG_OK;
}

extern "C" int sg_engine_timing(sg_ctx* c, double* t) {
  if (!c || !t) return SG_ERR_INVALID;
  const Engine& e = c->eng;
  t[0] = e.t_step_ms;
  t[1] = e.t_gemm_ms;
  t[2] = e.gemm_launches;
  t[3] = e.gemm_flops;
  t[4] = e.gemm_cols;
  t[5] = e.useful_cols;
  return SG_OK;
}

extern "C" int sg_engine_idle_ms(sg_ctx* c, double* ms) {
  if (!c || !ms) return SG_ERR_INVALID;
  ms[0] = c->eng.t_idle_ms;
  ms[1] = c->eng.t_admit_ms;
  ms[2] = c->eng.t_finish_host_ms;
  return SG_OK;
}

extern "C" int sg_engine_reset_timing(sg_ctx* c) {
  if (!c) return SG_ERR_INVALID;
  Engine& e = c->eng;
  e.t_idle_ms = 0.0;
  e.t_admit_ms = 0.0;
  e.t_finish_host_ms = 0.0;
  e.have_prev = false;
  e.have_fin_end = false;
  e.t_step_ms = e.t_gemm_ms = e.gemm_launches = e.gemm_flops = e.gemm_cols = e.useful_cols = 0;
  e.io_h2d = e.io_d2h = 0;
  e.trace.clear();
  return SG_OK;
}

extern "C" int sg_engine_step_trace(sg_ctx* c, double* out, int64_t max_steps, int64_t* n_out) {
  if (!c || !n_out || (max_steps > 0 && !out)) return SG_ERR_INVALID;
  const std::vector<double>& t = c->eng.trace;
  const int64_t n = std::min<int64_t>(max_steps, (int64_t)t.size() / kTraceFields);
  std::copy(t.begin(), t.begin() + n * kTraceFields, out);
  *n_out = n;
  return SG_OK;
}

extern "C" int sg_engine_io_bytes(sg_ctx* c, uint64_t* h2d_bytes, uint64_t* d2h_bytes) {
  if (!c || !h2d_bytes || !d2h_bytes) return SG_ERR_INVALID;
  *h2d_bytes = c->eng.io_h2d;
  *d2h_bytes = c->eng.io_d2h;
  return SG_OK;
}

extern "C" int sg_engine_stats(sg_ctx* c, int64_t* s4) {
  if (!c || !s4) return SG_ERR_INVALID;
  s4[0] = c->eng.steps;
  s4[1] = c->eng.retired;
  s4[2] = c->eng.col_iters;
  s4[3] = c->eng.grm_passes;
  return SG_OK;
}

// ------------------------------------------------------------------ leave one chromosome out
static void loco_free(sg_ctx* c) {
  dev_free_t(c, c->d_diag_loco);
  dev_free_t(c, c->d_zm);
  dev_free_t(c, c->d_zs);
  dev_free_t(c, c->d_lu);
  dev_free_t(c, c->d_lv);
  dev_free_t(c, c->d_lp);
  c->loco = false;
  c->loco_mj = c->loco_mjp = 0;
}

// Y <- (M Y - Z_j (Z_j' P)) / (M - M_j): parallelCrossProd_LOCO (FIT.cpp:1790-1851) on the resident K.
static int loco_correct(sg_ctx* c, int64_t ncols, bool yf) {
  Engine& e = c->eng;
  if (!c->d_lu) SG_TRY(dev_alloc_t(c, &c->d_lu, (size_t)(e.cap_cols * c->loco_mjp)));
  if (!c->d_lv) SG_TRY(dev_alloc_t(c, &c->d_lv, (size_t)(e.cap_cols * e.np)));
  const int64_t nc = round_up(ncols, kRowTile);  // the SIMT GEMM's row tile; rows past ncols read zero Pf
  if (nc > e.cap_cols) return set_err(c, SG_ERR_STATE, "LOCO needs engine capacity in multiples of 128 columns");
  // the correction needs P in full FP32: the split engine keeps P = Pf (tf32 high) + Pflo, the
  // plain FP64 engine keeps P in FP64
  const float* P = e.Pf;
  if (c->mv_mode == SG_MV_FP64_PLAIN || c->mv_mode == SG_MV_TF32X3_TC) {
    if (!c->d_lp) {
      SG_TRY(dev_alloc_t(c, &c->d_lp, (size_t)(e.cap_cols * e.np)));
      SG_CUDA(c, cudaMemsetAsync(c->d_lp, 0, (size_t)(e.cap_cols * e.np) * 4, c->stream));
    }
    if (c->mv_mode == SG_MV_FP64_PLAIN) {
      launch_f64_to_f32(e.P, c->d_lp, ncols * e.np, c->stream);
    } else {
      SG_CUDA(c, cudaMemcpyAsync(c->d_lp, e.Pf, ncols * e.np * 4, cudaMemcpyDeviceToDevice, c->stream));
      add_inplace_kernel<<<(unsigned)((ncols * e.np + 255) / 256), 256, 0, c->stream>>>(c->d_lp, e.Pflo, ncols * e.np);
    }
    c->launches += 1;
    P = c->d_lp;
  }
  // U (nc x mjp) = P Z_j' ; V (ncols x np, stored transposed) = Z_j U'
  launch_gemm_nt_f32(P, e.np, c->d_zm, e.np, c->d_lu, c->loco_mjp, nc, c->loco_mjp, e.np, 1.0f, 0, c->stream);
  launch_gemm_nt_f32(c->d_zs, c->loco_mjp, c->d_lu, c->loco_mjp, c->d_lv, e.np, e.np, ncols, c->loco_mjp, 1.0f, 1, c->stream);
  const double M = (double)c->m_qc;
  launch_loco_combine(yf ? e.Yf : nullptr, yf ? nullptr : e.Yd, c->d_lv, M, 1.0 / (M - (double)c->loco_mj),
                      ncols * e.np, c->stream);
  SG_LAUNCHED(c, 3);
  return SG_OK;
}

extern "C" int sg_loco_set(sg_ctx* c, int64_t begin, int64_t end) {
  NEED_GRM(c);
  if (begin < 0 || end < begin || end >= c->m_qc)
    return set_err(c, SG_ERR_INVALID, "LOCO range [%lld, %lld] outside the %lld GRM markers", (long long)begin,
                   (long long)end, (long long)c->m_qc);
  if (end - begin + 1 >= c->m_qc) return set_err(c, SG_ERR_INVALID, "LOCO range covers every GRM marker");
  if (exact_mode(c->mv_mode))
    return set_err(c, SG_ERR_STATE, "the subset-exact engines leave out .bim markers (sg_loco_set_bim)");
  for (auto& kv : c->eng.reqs)
    if (kv.second.state == 1) return set_err(c, SG_ERR_STATE, "columns in flight");
  loco_free(c);
  const int64_t mj = end - begin + 1;
  const int64_t mjp = round_up(mj, kRowTile);
  const int64_t np = c->np;
  SG_TRY(dev_alloc_t(c, &c->d_zm, (size_t)(mjp * np)));
  SG_TRY(dev_alloc_t(c, &c->d_zs, (size_t)(np * mjp)));
  const uint8_t* pk = c->d_packed + begin * c->pitch;
  const float* lut = c->d_lut + 4 * begin;
  launch_zbuild_marker_major(pk, c->pitch, lut, mj, mjp, c->nn, np, c->d_zm, c->stream);
  launch_zbuild_f32(pk, c->pitch, lut, mj, c->nn, np, mjp, c->d_zs, c->stream);
  // the chromosome's diagonal contribution (set_Diagof_StdGeno_LOCO, FIT.cpp:4934-4959)
  double* dj = nullptr;
  float* dj32 = nullptr;
  void* lutq = nullptr;
  SG_TRY(dev_alloc_t(c, &dj, (size_t)c->nn));
  SG_TRY(dev_alloc_t(c, &dj32, (size_t)c->nn));
  SG_TRY(dev_alloc(c, &lutq, (size_t)(48 * mj)));
  // the cohort's fractional bits bound this subset's sum too
  launch_diag(pk, c->pitch, lut, mj, c->nn, c->diag_frac_bits, lutq, dj, dj32, c->stream);
  SG_LAUNCHED(c, 4);
  std::vector<double> h(c->nn);
  SG_CUDA(c, cudaMemcpyAsync(h.data(), dj, c->nn * 8, cudaMemcpyDeviceToHost, c->stream));
  SG_TRY(sync(c));
  dev_free(c, dj);
  dev_free(c, dj32);
  dev_free(c, lutq);
  c->diag_loco.resize(c->nn);
  for (int64_t i = 0; i < c->nn; ++i) c->diag_loco[i] = c->diag[i] - h[i];
  SG_TRY(dev_alloc_t(c, &c->d_diag_loco, (size_t)c->nn));
  SG_CUDA(c, cudaMemcpy(c->d_diag_loco, c->diag_loco.data(), c->nn * 8, cudaMemcpyHostToDevice));
  c->loco_begin = begin;
  c->loco_end = end;
  c->loco_mj = mj;
  c->loco_mjp = mjp;
  c->loco = true;
  return SG_OK;
}

// One chromosome as .bim markers [begin, end].  On a resident GRM it is the range of GRM markers
// inside it (the GRM markers are the .bim markers passing QC, in order); in the subset-exact engines
// each phenotype's GRM markers are those passing QC over its own samples, so every slot's subset
// state leaves out its own GRM markers inside [begin, end] when the slot is next set.
extern "C" int sg_loco_set_bim(sg_ctx* c, int64_t begin, int64_t end) {
  NEED_GENO(c);
  if (begin < 0 || end < begin || end >= c->m_bim)
    return set_err(c, SG_ERR_INVALID, "LOCO range [%lld, %lld] outside the %lld .bim markers", (long long)begin,
                   (long long)end, (long long)c->m_bim);
  for (auto& kv : c->eng.reqs)
    if (kv.second.state == 1) return set_err(c, SG_ERR_STATE, "columns in flight");
  if (exact_mode(c->mv_mode)) {
    c->sub_loco_lo = begin;
    c->sub_loco_hi = end;
    return SG_OK;
  }
  int64_t b = 0;
  for (int64_t i = 0; i < begin; ++i) b += c->qc_mask[i] ? 1 : 0;
  int64_t e = b - 1;
  for (int64_t i = begin; i <= end; ++i) e += c->qc_mask[i] ? 1 : 0;
  if (e < b) return set_err(c, SG_ERR_INVALID, "no GRM marker in .bim markers [%lld, %lld]", (long long)begin, (long long)end);
  return sg_loco_set(c, b, e);
}

extern "C" int sg_loco_clear(sg_ctx* c) {
  if (!c) return SG_ERR_INVALID;
  for (auto& kv : c->eng.reqs)
    if (kv.second.state == 1) return set_err(c, SG_ERR_STATE, "columns in flight");
  loco_free(c);
  c->sub_loco_lo = 0;
  c->sub_loco_hi = -1;
  return SG_OK;
}

// ------------------------------------------------------------------ drop-in helpers (FP64 host LA)
namespace {

// run the engine until every id in ``ids`` has finished
int run_until(sg_ctx* c, const std::vector<int64_t>& ids) {
  Engine& e = c->eng;
  for (;;) {
    bool all = true;
    for (int64_t id : ids) {
      auto it = e.reqs.find(id);
      if (it != e.reqs.end() && it->second.state != 2) { all = false; break; }
    }
    if (all) return SG_OK;
    int64_t fin = 0;
    const int64_t before = e.steps;
    SG_TRY(sg_engine_run(c, 1 << 20, &fin));
    if (fin == 0 && e.steps == before)
      return set_err(c, SG_ERR_STATE, "engine made no progress with unfinished requests");
  }
}

int fetch(sg_ctx* c, int64_t id, double* x, int32_t* it) { return sg_engine_fetch(c, id, x, it); }

// Drop-ins run on phenotype slot 0 with capacity for one probe block.
int dropin_setup(sg_ctx* c, const float* w, const float* tau, int64_t cols) {
  NEED_OPERATOR(c);
  Engine& e = c->eng;
  SG_TRY(engine_clear(c));
  if (e.cap_cols < cols || e.cap_ph < 1 || e.np != c->np) SG_TRY(engine_reserve(c, std::max<int64_t>(cols, 128), 1));
  std::vector<double> wd(c->nn);
  for (int64_t i = 0; i < c->nn; ++i) wd[i] = w[i];
  const double td[2] = {tau[0], tau[1]};
  return sg_engine_set_pheno(c, 0, wd.data(), td, nullptr);
}

void f2d(const float* a, int64_t n, std::vector<double>& out) {
  out.resize(n);
  for (int64_t i = 0; i < n; ++i) out[i] = a[i];
}


// P v = Sv - SX cov (SX' v) with SX n x p (column-major), cov p x p
void p_apply(int64_t n, int p, const double* Sv, const double* SX, const double* cov, const double* v,
             double* out) {
  std::vector<double> t(p, 0.0), u(p, 0.0);
  for (int j = 0; j < p; ++j) {
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) s += SX[i + j * n] * v[i];
    t[j] = s;
  }
  for (int i = 0; i < p; ++i) {
    double s = 0.0;
    for (int j = 0; j < p; ++j) s += cov[i + j * p] * t[j];
    u[i] = s;
  }
  for (int64_t i = 0; i < n; ++i) {
    double s = 0.0;
    for (int j = 0; j < p; ++j) s += SX[i + j * n] * u[j];
    out[i] = Sv[i] - s;
  }
}

double dot(int64_t n, const double* a, const double* b) {
  double s = 0.0;
  for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

double cal_cv(const std::vector<double>& x) {
  const int64_t n = (int64_t)x.size();
  double m = 0.0;
  for (double v : x) m += v;
  m /= n;
  double ss = 0.0;
  for (double v : x) ss += (v - m) * (v - m);
  const double sd = std::sqrt(ss / (n - 1));
  return (sd / m) / n;
}

struct TraceOut {
  double tr1 = 0.0, tr0 = 0.0;
  int nrun = 0;
};

// tr(PK)_j = Au.Su - b' cov c and tr(P)_j = u.Su - c' cov c from the device-side probe dots
// (b_q = Au.SX_q, c_q = SX_q.u); appends to t1 / t0.  Errors land in c->err_pending.
void probe_terms(sg_ctx* c, const std::vector<int64_t>& pid, const std::vector<int64_t>& aid,
                 uint64_t seed, int64_t run0, const std::vector<double>& SX, int p,
                 const std::vector<double>& cov, std::vector<double>& t1, std::vector<double>& t0) {
  const int64_t k = (int64_t)pid.size(), nv = 2 + 2 * p;
  std::vector<double> D(k * nv);
  c->err_pending.clear();
  if (sg_engine_probe_dots(c, 0, pid.data(), aid.data(), k, seed, run0, SX.data(), p, D.data(), nullptr) != SG_OK) {
    c->err_pending = c->err;
    return;
  }
  for (int64_t j = 0; j < k; ++j) {
    const double* d = &D[j * nv];
    double bcb = 0.0, ccc = 0.0;
    for (int a = 0; a < p; ++a)
      for (int b = 0; b < p; ++b) {
        bcb += d[2 + a] * cov[a + b * p] * d[2 + p + b];
        ccc += d[2 + p + a] * cov[a + b * p] * d[2 + p + b];
      }
    t1.push_back(d[0] - bcb);
    t0.push_back(d[1] - ccc);
  }
}

// GetTrace / GetTrace_q on the engine: each block of probes is submitted as
// PCG columns (Sigma^-1 u) and product columns (K u) together.
int trace_probes(sg_ctx* c, const std::vector<double>& SX, int p, const std::vector<double>& cov,
                 int nrun, int maxiter, double tol, double cutoff, uint64_t seed, bool quant,
                 const std::vector<int64_t>& extra_ids, TraceOut* out) {
  Engine& e = c->eng;
  std::vector<double> t1, t0;
  int start = 0, end = nrun;
  bool first = true;
  e.hold = true;  // probe results are reduced on the device (sg_engine_probe_dots)
  for (;;) {
    const int k = end - start;
    std::vector<int64_t> pid(k), aid(k);
    SG_TRY(sg_engine_submit_probes(c, 0, 0, seed, start, k, maxiter, tol, pid.data()));
    SG_TRY(sg_engine_submit_probes(c, 0, 1, seed, start, k, maxiter, tol, aid.data()));
    std::vector<int64_t> all(pid);
    all.insert(all.end(), aid.begin(), aid.end());
    if (first) all.insert(all.end(), extra_ids.begin(), extra_ids.end());
    first = false;
    SG_TRY(run_until(c, all));
    probe_terms(c, pid, aid, seed, start, SX, p, cov, t1, t0);
    if (!c->err_pending.empty()) { e.hold = false; return set_err(c, SG_ERR_CUDA, "%s", c->err_pending.c_str()); }
    const double cv1 = cal_cv(t1);
    const double cv0 = quant ? cal_cv(t0) : 0.0;
    if (cv1 > cutoff || (quant && cv0 > cutoff)) {
      start = end;
      end += 10;
      continue;
    }
    break;
  }
  e.hold = false;
  double s1 = 0.0, s0 = 0.0;
  for (double v : t1) s1 += v;
  for (double v : t0) s0 += v;
  out->tr1 = s1 / t1.size();
  out->tr0 = s0 / t0.size();
  out->nrun = (int)t1.size();
  return SG_OK;
}

}  // namespace

// ------------------------------------------------------------------ drop-ins
extern "C" int sg_grm_matmul(sg_ctx* c, const double* V, int64_t k, double* out) {
  NEED_OPERATOR(c);
  if (k <= 0 || !V || !out) return set_err(c, SG_ERR_INVALID, "bad arguments");
  {
    std::vector<float> w(c->nn, 1.0f);
    const float tau[2] = {1.0f, 0.0f};
    SG_TRY(dropin_setup(c, w.data(), tau, std::min<int64_t>(k, 256)));
  }
  std::vector<int64_t> ids(k);
  SG_TRY(sg_engine_submit(c, 0, 1, V, k, 1, 0.0, ids.data()));
  SG_TRY(run_until(c, ids));
  for (int64_t j = 0; j < k; ++j) SG_TRY(fetch(c, ids[j], out + j * c->nn, nullptr));
  return SG_OK;
}

extern "C" int sg_getCrossprodMatAndKin(sg_ctx* c, const float* b, float* out) {
  NEED_OPERATOR(c);
  std::vector<double> bd, od(c->nn);
  f2d(b, c->nn, bd);
  SG_TRY(sg_grm_matmul(c, bd.data(), 1, od.data()));
  for (int64_t i = 0; i < c->nn; ++i) out[i] = (float)od[i];
  return SG_OK;
}

extern "C" int sg_getDiagOfSigma(sg_ctx* c, const float* w, const float* tau, float* out) {
  NEED_GENO(c);
  // float arithmetic in the reference's order: (tau1 * diag) / M + tau0 / w, floored at 1e-4
  const float M = (float)c->m_qc;
  for (int64_t i = 0; i < c->nn; ++i) {
    float v = c->is_diag_one ? tau[1] + tau[0] / w[i] : (tau[1] * c->diag32[i]) / M + tau[0] / w[i];
    out[i] = v < 1e-4f ? 1e-4f : v;
  }
  return SG_OK;
}

extern "C" int sg_getCrossprod(sg_ctx* c, const float* b, const float* w, const float* tau, float* out) {
  NEED_OPERATOR(c);
  const int64_t n = c->nn;
  if (tau[1] == 0.0f) {
    for (int64_t i = 0; i < n; ++i) out[i] = tau[0] * (b[i] * (1.0f / w[i]));
    return SG_OK;
  }
  std::vector<float> kb(n);
  SG_TRY(sg_getCrossprodMatAndKin(c, b, kb.data()));
  for (int64_t i = 0; i < n; ++i) out[i] = tau[0] * (b[i] * (1.0f / w[i])) + tau[1] * kb[i];
  return SG_OK;
}

extern "C" int sg_pcg_solve(sg_ctx* c, const double* w, const double* tau, const double* B, int64_t k,
                            int maxiter, double tol, double* X, int32_t* iters) {
  NEED_OPERATOR(c);
  if (k <= 0 || !w || !tau || !B || !X) return set_err(c, SG_ERR_INVALID, "bad arguments");
  Engine& e = c->eng;
  SG_TRY(engine_clear(c));
  if (e.cap_cols < std::min<int64_t>(k, 256) || e.cap_ph < 1 || e.np != c->np)
    SG_TRY(engine_reserve(c, std::min<int64_t>(std::max<int64_t>(k, 128), 2048), 1));
  SG_TRY(sg_engine_set_pheno(c, 0, w, tau, nullptr));
  std::vector<int64_t> ids(k);
  SG_TRY(sg_engine_submit(c, 0, 0, B, k, maxiter, tol, ids.data()));
  SG_TRY(run_until(c, ids));
  for (int64_t j = 0; j < k; ++j) SG_TRY(fetch(c, ids[j], X + j * c->nn, iters ? iters + j : nullptr));
  return SG_OK;
}

static int solve_f32(sg_ctx* c, const float* w, const float* tau, const float* B, int64_t k, int maxiter,
                     float tol, float* out, int32_t* iters) {
  NEED_OPERATOR(c);
  const int64_t n = c->nn;
  if (!all_finite(w, n) || !all_finite(tau, 2)) return set_err(c, SG_ERR_NUMERIC, "W or tau not finite");
  std::vector<double> wd, bd, xd(n * k);
  f2d(w, n, wd);
  f2d(B, n * k, bd);
  const double td[2] = {tau[0], tau[1]};
  SG_TRY(sg_pcg_solve(c, wd.data(), td, bd.data(), k, maxiter, (double)tol, xd.data(), iters));
  for (int64_t i = 0; i < n * k; ++i) out[i] = (float)xd[i];
  return SG_OK;
}

extern "C" int sg_getPCG1ofSigmaAndVector(sg_ctx* c, const float* w, const float* tau, const float* b,
                                          int maxiter, float tol, float* out, int32_t* iters) {
  return solve_f32(c, w, tau, b, 1, maxiter, tol, out, iters);
}
extern "C" int sg_getSigma_X(sg_ctx* c, const float* w, const float* tau, const float* X, int64_t p,
                             int maxiter, float tol, float* out) {
  return solve_f32(c, w, tau, X, p, maxiter, tol, out, nullptr);
}
extern "C" int sg_getSigma_G(sg_ctx* c, const float* w, const float* tau, const float* g, int maxiter,
                             float tol, float* out) {
  return solve_f32(c, w, tau, g, 1, maxiter, tol, out, nullptr);
}

extern "C" int sg_getCoefficients(sg_ctx* c, const float* Y, const float* X, int64_t p, const float* w,
                                  const float* tau, int maxiter, float tol, float* Sigma_iY,
                                  float* Sigma_iX, float* cov, float* alpha, float* eta) {
  NEED_OPERATOR(c);
  const int64_t n = c->nn;
  if (p <= 0) return set_err(c, SG_ERR_INVALID, "p must be positive");
  std::vector<float> B(n * (p + 1));
  std::copy(Y, Y + n, B.begin());
  std::copy(X, X + n * p, B.begin() + n);
  std::vector<float> S(n * (p + 1));
  SG_TRY(solve_f32(c, w, tau, B.data(), p + 1, maxiter, tol, S.data(), nullptr));
  std::vector<double> SY(n), SX(n * p), Xd, Yd;
  for (int64_t i = 0; i < n; ++i) SY[i] = S[i];
  for (int64_t i = 0; i < n * p; ++i) SX[i] = S[n + i];
  f2d(X, n * p, Xd);
  f2d(Y, n, Yd);
  std::vector<double> XtSX(p * p);
  for (int a = 0; a < p; ++a)
    for (int b = 0; b < p; ++b) XtSX[a + b * p] = dot(n, &Xd[a * n], &SX[b * n]);
  std::vector<double> cv = inv_sympd(XtSX, (int)p);
  std::vector<double> sxy(p), al(p, 0.0);
  for (int j = 0; j < p; ++j) sxy[j] = dot(n, &SX[j * n], Yd.data());
  for (int i = 0; i < p; ++i)
    for (int j = 0; j < p; ++j) al[i] += cv[i + j * p] * sxy[j];
  for (int64_t i = 0; i < n; ++i) {
    double sxa = 0.0;
    for (int j = 0; j < p; ++j) sxa += SX[i + j * n] * al[j];
    eta[i] = (float)(Yd[i] - (double)tau[0] * (SY[i] - sxa) / (double)w[i]);
    Sigma_iY[i] = (float)SY[i];
  }
  for (int64_t i = 0; i < n * p; ++i) Sigma_iX[i] = (float)SX[i];
  for (int64_t i = 0; i < p * p; ++i) cov[i] = (float)cv[i];
  for (int64_t i = 0; i < p; ++i) alpha[i] = (float)al[i];
  return SG_OK;
}

static int trace_common(sg_ctx* c, const float* Sigma_iX, int64_t p, const float* w, const float* tau,
                        const float* cov, int nrun, int maxiter, float tol, float cutoff, uint64_t seed,
                        bool quant, float* trace, int32_t* nrun_used) {
  NEED_OPERATOR(c);
  if (nrun < 2) return set_err(c, SG_ERR_INVALID, "nrun must be >= 2");
  SG_TRY(dropin_setup(c, w, tau, 2 * nrun + 4));
  std::vector<double> SX, cv;
  f2d(Sigma_iX, c->nn * p, SX);
  f2d(cov, p * p, cv);
  TraceOut t;
  SG_TRY(trace_probes(c, SX, (int)p, cv, nrun, maxiter, tol, cutoff, seed, quant, {}, &t));
  if (quant) {
    trace[0] = (float)t.tr0;
    trace[1] = (float)t.tr1;
  } else {
    trace[0] = (float)t.tr1;
  }
  if (nrun_used) *nrun_used = t.nrun;
  return SG_OK;
}

extern "C" int sg_GetTrace(sg_ctx* c, const float* Sigma_iX, const float* X, int64_t p, const float* w,
                           const float* tau, const float* cov, int nrun, int maxiter, float tol,
                           float cutoff, uint64_t seed, float* trace, int32_t* nrun_used) {
  (void)X;
  return trace_common(c, Sigma_iX, p, w, tau, cov, nrun, maxiter, tol, cutoff, seed, false, trace, nrun_used);
}
extern "C" int sg_GetTrace_q(sg_ctx* c, const float* Sigma_iX, const float* X, int64_t p, const float* w,
                             const float* tau, const float* cov, int nrun, int maxiter, float tol,
                             float cutoff, uint64_t seed, float* trace, int32_t* nrun_used) {
  (void)X;
  return trace_common(c, Sigma_iX, p, w, tau, cov, nrun, maxiter, tol, cutoff, seed, true, trace, nrun_used);
}

namespace {
struct AIOut {
  double YPAPY = 0, YPA0PY = 0, tr0 = 0, tr1 = 0;
  double AI[4] = {0, 0, 0, 0};
  std::vector<double> PY;
};

// getAIScore / getAIScore_q: K PY rides with the first probe block; the
// P A PY (and P A0 PY) solves are submitted as soon as K PY is known.
int ai_score(sg_ctx* c, const float* Y, const float* X, int64_t p, const float* w, const float* tau,
             const float* Sigma_iY, const float* Sigma_iX, const float* cov_in, int nrun, int maxiter,
             float tol, float cutoff, uint64_t seed, bool quant, AIOut* o) {
  NEED_OPERATOR(c);
  const int64_t n = c->nn;
  SG_TRY(dropin_setup(c, w, tau, 2 * nrun + 8));
  std::vector<double> Yd, Xd, SY, SX, cv;
  f2d(Y, n, Yd);
  f2d(X, n * p, Xd);
  f2d(Sigma_iY, n, SY);
  f2d(Sigma_iX, n * p, SX);
  if (quant) {
    std::vector<double> XtSX(p * p);
    for (int a = 0; a < p; ++a)
      for (int b = 0; b < p; ++b) XtSX[a + b * p] = dot(n, &Xd[a * n], &SX[b * n]);
    cv = inv_sympd(XtSX, (int)p);
  } else {
    f2d(cov_in, p * p, cv);
  }
  o->PY.resize(n);
  p_apply(n, (int)p, SY.data(), SX.data(), cv.data(), Yd.data(), o->PY.data());
  c->eng.hold = true;  // probe results are reduced on the device
  int64_t apy_id;
  SG_TRY(sg_engine_submit(c, 0, 1, o->PY.data(), 1, 1, 0.0, &apy_id));
  // first probe block + K PY in the same steps
  const int k = nrun;
  std::vector<int64_t> pid(k), aid(k);
  SG_TRY(sg_engine_submit_probes(c, 0, 0, seed, 0, k, maxiter, tol, pid.data()));
  SG_TRY(sg_engine_submit_probes(c, 0, 1, seed, 0, k, maxiter, tol, aid.data()));
  SG_TRY(run_until(c, {apy_id}));
  std::vector<double> APY(n);
  SG_TRY(fetch(c, apy_id, APY.data(), nullptr));
  o->YPAPY = dot(n, o->PY.data(), APY.data());
  o->YPA0PY = dot(n, o->PY.data(), o->PY.data());
  std::vector<double> rhs(APY);
  int nsolve = 1;
  if (quant) {
    rhs.insert(rhs.end(), o->PY.begin(), o->PY.end());  // A0 PY = PY
    nsolve = 2;
  }
  std::vector<int64_t> sid(nsolve);
  SG_TRY(sg_engine_submit(c, 0, 0, rhs.data(), nsolve, maxiter, tol, sid.data()));
  // finish the first probe block (and the solves), then continue GetTrace's CV loop
  std::vector<int64_t> all(pid);
  all.insert(all.end(), aid.begin(), aid.end());
  all.insert(all.end(), sid.begin(), sid.end());
  SG_TRY(run_until(c, all));
  std::vector<double> t1, t0;
  probe_terms(c, pid, aid, seed, 0, SX, (int)p, cv, t1, t0);
  if (!c->err_pending.empty()) { c->eng.hold = false; return set_err(c, SG_ERR_CUDA, "%s", c->err_pending.c_str()); }
  int start = k, end = k;
  while (cal_cv(t1) > cutoff || (quant && cal_cv(t0) > cutoff)) {
    start = end;
    end = start + 10;
    std::vector<int64_t> p2(10), a2(10);
    SG_TRY(sg_engine_submit_probes(c, 0, 0, seed, start, 10, maxiter, tol, p2.data()));
    SG_TRY(sg_engine_submit_probes(c, 0, 1, seed, start, 10, maxiter, tol, a2.data()));
    std::vector<int64_t> al(p2);
    al.insert(al.end(), a2.begin(), a2.end());
    SG_TRY(run_until(c, al));
    probe_terms(c, p2, a2, seed, start, SX, (int)p, cv, t1, t0);
    if (!c->err_pending.empty()) { c->eng.hold = false; return set_err(c, SG_ERR_CUDA, "%s", c->err_pending.c_str()); }
  }
  c->eng.hold = false;
  double s1 = 0, s0 = 0;
  for (double v : t1) s1 += v;
  for (double v : t0) s0 += v;
  o->tr1 = s1 / t1.size();
  o->tr0 = s0 / t0.size();
  std::vector<double> S(n), PAPY(n);
  SG_TRY(fetch(c, sid[0], S.data(), nullptr));
  // the reference projects the solved vector: PAPY_1 - Sigma_iX cov (Sigma_iX' PAPY_1)
  // (FIT.cpp:3290-3291; 3507-3508 and 3513-3514 in the _q form)
  p_apply(n, (int)p, S.data(), SX.data(), cv.data(), S.data(), PAPY.data());
  o->AI[3] = dot(n, APY.data(), PAPY.data());
  if (quant) {
    std::vector<double> PA0PY(n);
    SG_TRY(fetch(c, sid[1], S.data(), nullptr));
    p_apply(n, (int)p, S.data(), SX.data(), cv.data(), S.data(), PA0PY.data());
    o->AI[0] = dot(n, o->PY.data(), PA0PY.data());
    o->AI[1] = o->AI[2] = dot(n, o->PY.data(), PAPY.data());
  }
  return SG_OK;
}
}  // namespace

extern "C" int sg_getAIScore(sg_ctx* c, const float* Y, const float* X, int64_t p, const float* w,
                             const float* tau, const float* Sigma_iY, const float* Sigma_iX,
                             const float* cov, int nrun, int maxiter, float tol, float cutoff,
                             uint64_t seed, float* YPAPY, float* Trace, float* AI, float* PY) {
  AIOut o;
  SG_TRY(ai_score(c, Y, X, p, w, tau, Sigma_iY, Sigma_iX, cov, nrun, maxiter, tol, cutoff, seed, false, &o));
  *YPAPY = (float)o.YPAPY;
  *Trace = (float)o.tr1;
  *AI = (float)o.AI[3];
  if (PY)
    for (int64_t i = 0; i < c->nn; ++i) PY[i] = (float)o.PY[i];
  return SG_OK;
}

extern "C" int sg_getAIScore_q(sg_ctx* c, const float* Y, const float* X, int64_t p, const float* w,
                               const float* tau, const float* Sigma_iY, const float* Sigma_iX,
                               const float* cov, int nrun, int maxiter, float tol, float cutoff,
                               uint64_t seed, float* YPAPY, float* YPA0PY, float* Trace, float* AI,
                               float* PY) {
  AIOut o;
  SG_TRY(ai_score(c, Y, X, p, w, tau, Sigma_iY, Sigma_iX, cov, nrun, maxiter, tol, cutoff, seed, true, &o));
  *YPAPY = (float)o.YPAPY;
  *YPA0PY = (float)o.YPA0PY;
  Trace[0] = (float)o.tr0;
  Trace[1] = (float)o.tr1;
  for (int i = 0; i < 4; ++i) AI[i] = (float)o.AI[i];
  if (PY)
    for (int64_t i = 0; i < c->nn; ++i) PY[i] = (float)o.PY[i];
  return SG_OK;
}

extern "C" int sg_fitglmmaiRPCG(sg_ctx* c, const float* Y, const float* X, int64_t p, const float* w,
                                float* tau, const float* Sigma_iY, const float* Sigma_iX, const float* cov,
                                int nrun, int maxiter, float tol_pcg, float tol, float cutoff,
                                uint64_t seed) {
  AIOut o;
  SG_TRY(ai_score(c, Y, X, p, w, tau, Sigma_iY, Sigma_iX, cov, nrun, maxiter, tol_pcg, cutoff, seed, false, &o));
  // FIT.cpp:3313-3337
  const double dtau = (o.YPAPY - o.tr1) / o.AI[3];
  const double t0[2] = {tau[0], tau[1]};
  double t[2] = {t0[0], t0[1] + dtau};
  for (double& v : t) if (v < tol) v = 0.0;
  double step = 1.0;
  while (t[1] < 0.0) {
    step *= 0.5;
    t[1] = t0[1] + step * dtau;
  }
  for (double& v : t) if (v < tol) v = 0.0;
  tau[0] = (float)t[0];
  tau[1] = (float)t[1];
  return SG_OK;
}

extern "C" int sg_fitglmmaiRPCG_q(sg_ctx* c, const float* Y, const float* X, int64_t p, const float* w,
                                  float* tau, const float* Sigma_iY, const float* Sigma_iX,
                                  const float* cov, int nrun, int maxiter, float tol_pcg, float tol,
                                  float cutoff, uint64_t seed) {
  AIOut o;
  SG_TRY(ai_score(c, Y, X, p, w, tau, Sigma_iY, Sigma_iX, cov, nrun, maxiter, tol_pcg, cutoff, seed, true, &o));
  // FIT.cpp:3615-3660: Dtau = solve(AI, score), GMMAT zeroing, step-halving
  const double s0 = o.YPA0PY - o.tr0, s1 = o.YPAPY - o.tr1;
  const double det = o.AI[0] * o.AI[3] - o.AI[1] * o.AI[2];
  if (det == 0.0 || !std::isfinite(det)) return set_err(c, SG_ERR_NUMERIC, "singular AI matrix");
  const double d0 = (o.AI[3] * s0 - o.AI[2] * s1) / det;
  const double d1 = (o.AI[0] * s1 - o.AI[1] * s0) / det;
  const double t0[2] = {tau[0], tau[1]};
  const bool zero[2] = {t0[0] < tol, t0[1] < tol};
  double t[2] = {t0[0] + d0, t0[1] + d1};
  for (int i = 0; i < 2; ++i) if (zero[i] && t[i] < tol) t[i] = 0.0;
  double step = 1.0;
  while (t[0] < 0.0 || t[1] < 0.0) {
    step *= 0.5;
    t[0] = t0[0] + step * d0;
    t[1] = t0[1] + step * d1;
    for (int i = 0; i < 2; ++i) if (zero[i] && t[i] < tol) t[i] = 0.0;
  }
  for (double& v : t) if (v < tol) v = 0.0;
  tau[0] = (float)t[0];
  tau[1] = (float)t[1];
  return SG_OK;
}

// ------------------------------------------------------------------ synthetic cohorts
extern "C" int sg_synth_bed(sg_ctx* c, uint64_t seed, int64_t n, int64_t m, double miss_rate,
                            uint8_t** bed_dev, uint64_t* bed_len) {
  if (!c || n <= 0 || m <= 0 || miss_rate < 0 || miss_rate >= 1) return SG_ERR_INVALID;
  dev_free_t(c, c->d_synth);
  const uint64_t len = 3 + (uint64_t)((n + 3) / 4) * (uint64_t)m;
  SG_TRY(dev_alloc_t(c, &c->d_synth, (size_t)len));
  const uint8_t magic[3] = {0x6C, 0x1B, 0x01};
  SG_CUDA(c, cudaMemcpyAsync(c->d_synth, magic, 3, cudaMemcpyHostToDevice, c->stream));
  const uint32_t thr = (uint32_t)std::llround(miss_rate * 65536.0);
  launch_synth_bed(seed, n, m, thr, c->d_synth, c->stream);
  SG_LAUNCHED(c, 1);
  SG_TRY(sync(c));
  c->synth_len = len;
  if (bed_dev) *bed_dev = c->d_synth;
  if (bed_len) *bed_len = len;
  return SG_OK;
}

extern "C" int sg_synth_bed_to_host(sg_ctx* c, uint8_t* host, uint64_t len) {
  if (!c || !c->d_synth) return SG_ERR_STATE;
  if (len > c->synth_len) return set_err(c, SG_ERR_INVALID, "length beyond the synthetic image");
  SG_CUDA(c, cudaMemcpy(host, c->d_synth, len, cudaMemcpyDeviceToHost));
  return SG_OK;
}

extern "C" int sg_synth_genetic_value(sg_ctx* c, uint64_t seed, double* out) {
  NEED_GENO(c);
  double* d = nullptr;
  SG_TRY(dev_alloc_t(c, &d, (size_t)c->nn));
  launch_genetic_value(c->d_packed, c->pitch, c->d_lut, c->m_qc, c->nn, seed, d, c->stream);
  SG_LAUNCHED(c, 2);
  SG_CUDA(c, cudaMemcpyAsync(out, d, c->nn * 8, cudaMemcpyDeviceToHost, c->stream));
  SG_TRY(sync(c));
  dev_free(c, d);
  return SG_OK;
}
