// A CPU stand-in for the batched solve engine, for testing the native fit driver (csrc/fits.cu)
// without a GPU.  It implements the sg_engine_* calls the driver makes with the engine's
// documented semantics (include/saigegpu.h): phenotype slots, queued / running / finished request
// states, held results, the per-slot probe cache, probe reductions and launch / finish stepping,
// over a dense FP64 kinship matrix given at creation.  The PCG column update is the Jacobi-
// preconditioned loop of getPCG1ofSigmaAndVector (FIT.cpp:2593-2809) with the operator
// tau0 b / W + tau1 K b of getCrossprod (FIT.cpp:2397-2425) and the diagonal of getDiagOfSigma
// (FIT.cpp:2322-2365); probes are the counter-hash Rademacher vectors of the engine.
//
// Test infrastructure only: built by tests/test_native_driver_cpu.py together with fits.cu.
#include "../../include/saigegpu.h"

#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <set>
#include <string>
#include <thread>
#include <vector>

namespace {

uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
uint64_t hash3(uint64_t seed, uint64_t stream, uint64_t idx) {
  uint64_t h = mix64(seed ^ 0x5851F42D4C957F2Dull);
  h = mix64(h ^ (stream * 0x9E3779B97F4A7C15ull));
  return mix64(h ^ (idx * 0xD1B54A32D192ED03ull));
}

enum { Q_QUEUED = 0, Q_RUNNING = 1, Q_DONE = 2 };

struct Req {
  int64_t slot = 0;
  int kind = 0, maxiter = 0, iters = 0, state = Q_QUEUED;
  double tol = 0.0, rz = 0.0, sumr2 = 0.0;
  bool stop = false;  // the launched step ended this column
  int64_t src = -1;   // chained: the right-hand side is this request's result
  std::vector<double> b, x, r, z, p;
};

struct Slot {
  bool set = false;
  double tau[2] = {0, 0};
  std::vector<double> winv, minv;
  std::vector<uint8_t> mask;
  std::map<std::pair<uint64_t, int64_t>, std::vector<double>> cache;  // K u by (seed, run)
};

}  // namespace

struct sg_ctx {
  int64_t n = 0;
  std::vector<double> K, diag;  // n x n (symmetric; empty: K = diag(diag)), diag(Sigma) term of K
  int64_t cap_cols = 0, running_or_held = 0;
  std::vector<Slot> slots;
  std::map<int64_t, Req> reqs;
  std::deque<int64_t> queue;
  std::vector<int64_t> finished;
  int64_t next_id = 1;
  bool hold = false, inflight = false;
  int64_t steps = 0, retired = 0, col_iters = 0;
  // driver checks: subset preparations, highest slot index prepared or set, most slots with
  // requests outstanding at a launch
  int64_t prepares = 0, max_slot = -1, max_busy_slots = 0;
  double step_ms = 0.0;  // emulated device time of a step
  std::chrono::steady_clock::time_point step_end;
  std::string err;
};

namespace {

int fail(sg_ctx* c, int code, const std::string& m) {
  c->err = m;
  return code;
}

// K v restricted to the slot's samples (0 outside)
void kprod(const sg_ctx* c, const Slot& s, const std::vector<double>& v, std::vector<double>& out) {
  const int64_t n = c->n;
  out.assign(n, 0.0);
  for (int64_t i = 0; i < n; ++i) {
    if (!s.mask[i]) continue;
    if (c->K.empty()) {  // K = diag(diag): large cohorts at O(n) per product
      out[i] = c->diag[i] * v[i];
      continue;
    }
    const double* row = c->K.data() + i * n;
    double acc = 0.0;
    for (int64_t j = 0; j < n; ++j) acc += row[j] * v[j];
    out[i] = acc;
  }
}

double dot(const std::vector<double>& a, const std::vector<double>& b) {
  double s = 0.0;
  for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
  return s;
}

void admit(sg_ctx* c) {
  std::deque<int64_t> later;  // chained requests whose source has not finished, in order
  while (!c->queue.empty() && c->running_or_held < c->cap_cols) {
    const int64_t id = c->queue.front();
    c->queue.pop_front();
    auto it = c->reqs.find(id);
    if (it == c->reqs.end()) continue;  // cancelled while queued
    Req& q = it->second;
    if (q.src >= 0) {
      auto is = c->reqs.find(q.src);
      if (is == c->reqs.end() || is->second.state != Q_DONE) {
        later.push_back(id);
        continue;
      }
      q.b = is->second.x;
      q.src = -1;
    }
    const Slot& s = c->slots[q.slot];
    const int64_t n = c->n;
    q.state = Q_RUNNING;
    c->running_or_held += 1;
    q.x.assign(n, 0.0);
    q.r.assign(n, 0.0);
    q.z.assign(n, 0.0);
    for (int64_t i = 0; i < n; ++i) q.r[i] = s.mask[i] ? q.b[i] : 0.0;
    for (int64_t i = 0; i < n; ++i) q.z[i] = s.minv[i] * q.r[i];
    q.p = q.z;
    q.rz = dot(q.r, q.z);
    q.sumr2 = dot(q.r, q.r);
    q.iters = 0;
    q.stop = q.kind == 0 && !(q.sumr2 > q.tol && q.iters < q.maxiter);
  }
  c->queue.insert(c->queue.begin(), later.begin(), later.end());
}

// Before request id leaves: chained requests queued on it take its result, or are cancelled with
// it when it has none.
void detach(sg_ctx* c, int64_t id) {
  auto is = c->reqs.find(id);
  if (is == c->reqs.end()) return;
  std::vector<int64_t> gone;
  for (auto& kv : c->reqs) {
    Req& q = kv.second;
    if (q.src != id) continue;
    if (is->second.state == Q_DONE) {
      q.b = is->second.x;
      q.src = -1;
    } else {
      gone.push_back(kv.first);
    }
  }
  for (int64_t g : gone) c->reqs.erase(g);
}

// One PCG iteration (or the product) of a running column.
void step_col(sg_ctx* c, Req& q) {
  const Slot& s = c->slots[q.slot];
  const int64_t n = c->n;
  if (q.kind == 1) {
    kprod(c, s, q.b, q.x);
    for (int64_t i = 0; i < n; ++i)
      if (!s.mask[i]) q.x[i] = 0.0;
    q.iters = 1;
    q.stop = true;
    return;
  }
  std::vector<double> kp;
  if (s.tau[1] != 0.0) kprod(c, s, q.p, kp);
  std::vector<double> ap(n, 0.0);
  for (int64_t i = 0; i < n; ++i)
    ap[i] = s.mask[i] ? s.tau[0] * s.winv[i] * q.p[i] + (s.tau[1] != 0.0 ? s.tau[1] * kp[i] : 0.0) : 0.0;
  const double a = q.rz / dot(q.p, ap);
  for (int64_t i = 0; i < n; ++i) q.x[i] += a * q.p[i];
  for (int64_t i = 0; i < n; ++i) q.r[i] -= a * ap[i];
  for (int64_t i = 0; i < n; ++i) q.z[i] = s.minv[i] * q.r[i];
  const double rz1 = dot(q.z, q.r);
  const double bet = rz1 / q.rz;
  for (int64_t i = 0; i < n; ++i) q.p[i] = q.z[i] + bet * q.p[i];
  q.rz = rz1;
  q.iters += 1;
  q.sumr2 = dot(q.r, q.r);
  q.stop = !(q.sumr2 > q.tol && q.iters < q.maxiter);
}

void retire_stopped(sg_ctx* c, int64_t* fin) {
  for (auto& kv : c->reqs) {
    Req& q = kv.second;
    if (q.state != Q_RUNNING || !q.stop) continue;
    q.state = Q_DONE;
    c->finished.push_back(kv.first);
    c->retired += 1;
    *fin += 1;
  }
}

void wait_device(sg_ctx* c) {
  if (c->inflight) std::this_thread::sleep_until(c->step_end);
}

}  // namespace

extern "C" {

// K NULL: K = diag(diag)
int fake_ctx_create(int64_t n, const double* K, const double* diag, double step_ms, sg_ctx** out) {
  if (n <= 0 || !diag || !out) return SG_ERR_INVALID;
  sg_ctx* c = new sg_ctx();
  c->n = n;
  if (K) c->K.assign(K, K + n * n);
  c->diag.assign(diag, diag + n);
  c->step_ms = step_ms;
  *out = c;
  return SG_OK;
}

void fake_ctx_destroy(sg_ctx* c) { delete c; }

// running or held columns (a finished, held result keeps its column)
int64_t fake_columns_in_use(sg_ctx* c) { return c ? c->running_or_held : -1; }
int64_t fake_requests(sg_ctx* c) { return c ? (int64_t)c->reqs.size() : -1; }
void fake_slot_stats(sg_ctx* c, int64_t* out) {
  out[0] = c->prepares;
  out[1] = c->max_slot;
  out[2] = c->max_busy_slots;
}

const char* sg_last_error(const sg_ctx* c) { return c ? c->err.c_str() : "null context"; }
int sg_ctx_make_current(sg_ctx* c) { return c ? SG_OK : SG_ERR_INVALID; }

int sg_geno_dims(sg_ctx* c, int64_t* n, int64_t* m_total, int64_t* m_qc, int64_t* m_vr) {
  if (!c) return SG_ERR_INVALID;
  if (n) *n = c->n;
  if (m_total) *m_total = 0;
  if (m_qc) *m_qc = 0;
  if (m_vr) *m_vr = 0;
  return SG_OK;
}

int sg_engine_reserve(sg_ctx* c, int64_t max_columns, int64_t max_phenos) {
  if (!c || max_columns <= 0 || max_phenos <= 0) return SG_ERR_INVALID;
  if (!c->reqs.empty()) return fail(c, SG_ERR_STATE, "reserve with requests outstanding");
  c->cap_cols = max_columns;
  c->slots.assign(max_phenos, Slot());
  return SG_OK;
}

int sg_engine_hold_results(sg_ctx* c, int hold) {
  if (!c) return SG_ERR_INVALID;
  c->hold = hold != 0;
  return SG_OK;
}

int sg_engine_set_pheno(sg_ctx* c, int64_t slot, const double* w, const double* tau, const uint8_t* mask) {
  if (!c || !w || !tau) return SG_ERR_INVALID;
  if (slot < 0 || slot >= (int64_t)c->slots.size()) return fail(c, SG_ERR_INVALID, "slot out of range");
  // stricter than the engine: a queued column of the slot would also see the new weights
  for (const auto& kv : c->reqs)
    if (kv.second.slot == slot && kv.second.state != Q_DONE)
      return fail(c, SG_ERR_STATE, "phenotype slot has columns queued or in flight");
  Slot& s = c->slots[slot];
  c->max_slot = std::max(c->max_slot, slot);
  const int64_t n = c->n;
  s.mask.assign(n, 1);
  if (mask)
    for (int64_t i = 0; i < n; ++i) s.mask[i] = mask[i] ? 1 : 0;
  s.winv.assign(n, 0.0);
  s.minv.assign(n, 0.0);
  for (int64_t i = 0; i < n; ++i) {
    if (!s.mask[i]) continue;
    if (!(std::isfinite(w[i]) && w[i] > 0.0)) return fail(c, SG_ERR_NUMERIC, "W is not a positive finite weight");
    const double d = tau[1] * c->diag[i] + tau[0] / w[i];
    s.winv[i] = 1.0 / w[i];
    s.minv[i] = 1.0 / (d < 1e-4 ? 1e-4 : d);
  }
  s.tau[0] = tau[0];
  s.tau[1] = tau[1];
  s.set = true;
  return SG_OK;
}

static int submit_common(sg_ctx* c, int64_t slot, int kind, const double* B, bool probe, uint64_t seed,
                         int64_t run0, int64_t k, int maxiter, double tol, int64_t* ids) {
  if (!c) return SG_ERR_INVALID;
  if (slot < 0 || slot >= (int64_t)c->slots.size() || !c->slots[slot].set)
    return fail(c, SG_ERR_STATE, "phenotype slot not set");
  if (kind != 0 && kind != 1) return fail(c, SG_ERR_INVALID, "kind must be 0 or 1");
  const Slot& s = c->slots[slot];
  const int64_t n = c->n;
  for (int64_t j = 0; j < k; ++j) {
    Req q;
    q.slot = slot;
    q.kind = kind;
    q.maxiter = maxiter;
    q.tol = tol;
    q.b.assign(n, 0.0);
    for (int64_t i = 0; i < n; ++i) {
      if (probe)
        q.b[i] = s.mask[i] ? ((hash3(seed, (uint64_t)(run0 + j), (uint64_t)i) >> 63) ? 1.0 : -1.0) : 0.0;
      else
        q.b[i] = B[j * n + i];
    }
    const int64_t id = c->next_id++;
    if (ids) ids[j] = id;
    c->reqs.emplace(id, std::move(q));
    c->queue.push_back(id);
  }
  return SG_OK;
}

int sg_engine_submit(sg_ctx* c, int64_t slot, int kind, const double* B, int64_t k, int maxiter, double tol,
                     int64_t* ids) {
  return submit_common(c, slot, kind, B, false, 0, 0, k, maxiter, tol, ids);
}

int sg_engine_submit_probes(sg_ctx* c, int64_t slot, int kind, uint64_t seed, int64_t run0, int64_t k, int maxiter,
                            double tol, int64_t* ids) {
  return submit_common(c, slot, kind, nullptr, true, seed, run0, k, maxiter, tol, ids);
}

int sg_engine_submit_chained(sg_ctx* c, int64_t slot, const int64_t* src_ids, int64_t k, int maxiter, double tol,
                             int64_t* ids) {
  if (!c || k < 0 || (k > 0 && !src_ids)) return SG_ERR_INVALID;
  if (!c->hold) return fail(c, SG_ERR_STATE, "chained solves need held results");
  if (slot < 0 || slot >= (int64_t)c->slots.size() || !c->slots[slot].set)
    return fail(c, SG_ERR_STATE, "phenotype slot not set");
  for (int64_t j = 0; j < k; ++j)
    if (!c->reqs.count(src_ids[j])) return fail(c, SG_ERR_NOT_FOUND, "unknown source request");
  for (int64_t j = 0; j < k; ++j) {
    Req q;
    q.slot = slot;
    q.kind = 0;
    q.maxiter = maxiter;
    q.tol = tol;
    q.src = src_ids[j];
    const int64_t id = c->next_id++;
    if (ids) ids[j] = id;
    c->reqs.emplace(id, std::move(q));
    c->queue.push_back(id);
  }
  return SG_OK;
}

int sg_engine_launch(sg_ctx* c, int64_t* n_finished, int* launched) {
  if (!c) return SG_ERR_INVALID;
  if (c->inflight) return fail(c, SG_ERR_STATE, "a step is in flight: finish it first");
  if (n_finished) *n_finished = 0;
  if (launched) *launched = 0;
  {
    std::set<int64_t> busy;
    for (const auto& kv : c->reqs) busy.insert(kv.second.slot);
    c->max_busy_slots = std::max(c->max_busy_slots, (int64_t)busy.size());
  }
  admit(c);
  bool any = false;
  for (auto& kv : c->reqs) {
    Req& q = kv.second;
    if (q.state != Q_RUNNING) continue;
    any = true;
    if (q.stop) continue;  // converged at admission: retires with this step
    step_col(c, q);
    c->col_iters += 1;
  }
  if (!any) return SG_OK;
  c->inflight = true;
  c->step_end = std::chrono::steady_clock::now() + std::chrono::microseconds((int64_t)(c->step_ms * 1e3));
  if (launched) *launched = 1;
  return SG_OK;
}

int sg_engine_wait(sg_ctx* c) {
  if (!c) return SG_ERR_INVALID;
  wait_device(c);
  return SG_OK;
}

// the split probe reduction: _begin keeps the arguments, _end runs the whole reduction
struct FakeDots {
  std::vector<int64_t> pcg, prod;
  std::vector<double> sx;
  int64_t k = 0, p = 0, run0 = 0;
  uint64_t seed = 0;
  bool pending = false;
};
static std::map<std::pair<const sg_ctx*, int64_t>, FakeDots> g_fake_dots;

int sg_engine_probe_dots_begin(sg_ctx* c, int64_t slot, const int64_t* ids_pcg, const int64_t* ids_prod, int64_t k,
                               uint64_t seed, int64_t run0, const double* SX, int64_t p) {
  if (!c || k <= 0 || !ids_pcg || !ids_prod || p < 0 || p > 16 || (p > 0 && !SX))
    return fail(c, SG_ERR_INVALID, "probe_dots: bad arguments");
  FakeDots& d = g_fake_dots[{c, slot}];
  if (d.pending) return fail(c, SG_ERR_STATE, "probe reduction in flight");
  d.pcg.assign(ids_pcg, ids_pcg + k);
  d.prod.assign(ids_prod, ids_prod + k);
  d.sx.assign(SX ? SX : nullptr, SX ? SX + p * c->n : nullptr);
  d.k = k;
  d.p = p;
  d.seed = seed;
  d.run0 = run0;
  d.pending = true;
  return SG_OK;
}

int sg_engine_probe_dots_wait(sg_ctx* c, int64_t slot) {
  (void)slot;
  return c ? SG_OK : SG_ERR_INVALID;
}

int sg_engine_probe_dots_end(sg_ctx* c, int64_t slot, double* out, int32_t* iters) {
  if (!c) return SG_ERR_INVALID;
  auto it = g_fake_dots.find({c, slot});
  if (it == g_fake_dots.end() || !it->second.pending) return fail(c, SG_ERR_STATE, "no probe reduction in flight");
  FakeDots d = it->second;
  it->second.pending = false;
  return sg_engine_probe_dots(c, slot, d.pcg.data(), d.prod.data(), d.k, d.seed, d.run0,
                              d.p ? d.sx.data() : nullptr, d.p, out, iters);
}

// the fake keeps no subset state: preparing and waiting only check their arguments
int sg_engine_prepare_subset(sg_ctx* c, int64_t slot, const uint8_t* mask) {
  (void)mask;
  if (!c) return SG_ERR_INVALID;
  if (slot < 0 || slot >= (int64_t)c->slots.size()) return fail(c, SG_ERR_INVALID, "slot out of range");
  ++c->prepares;
  c->max_slot = std::max(c->max_slot, slot);
  return SG_OK;
}

int sg_engine_subset_wait(sg_ctx* c, int64_t slot) {
  (void)slot;
  return c ? SG_OK : SG_ERR_INVALID;
}

int sg_engine_finish(sg_ctx* c, int64_t* n_finished) {
  if (!c) return SG_ERR_INVALID;
  int64_t fin = 0;
  if (c->inflight) {
    wait_device(c);
    c->inflight = false;
    c->steps += 1;
    retire_stopped(c, &fin);
  }
  if (n_finished) *n_finished = fin;
  return SG_OK;
}

int sg_engine_run(sg_ctx* c, int64_t max_steps, int64_t* n_finished) {
  if (!c) return SG_ERR_INVALID;
  int64_t fin = 0;
  if (c->inflight) {
    sg_engine_finish(c, &fin);
    if (fin > 0 || max_steps <= 0) {
      if (n_finished) *n_finished = fin;
      return SG_OK;
    }
  }
  for (int64_t s = 0; s < max_steps && fin == 0; ++s) {
    int launched = 0;
    const int rc = sg_engine_launch(c, nullptr, &launched);
    if (rc != SG_OK) return rc;
    if (!launched) break;
    sg_engine_finish(c, &fin);
  }
  if (n_finished) *n_finished = fin;
  return SG_OK;
}

int sg_engine_fetch(sg_ctx* c, int64_t id, double* x, int32_t* iters) {
  if (!c) return SG_ERR_INVALID;
  auto it = c->reqs.find(id);
  if (it == c->reqs.end()) return fail(c, SG_ERR_NOT_FOUND, "unknown request");
  if (it->second.state != Q_DONE) return fail(c, SG_ERR_STATE, "request not finished");
  detach(c, id);
  if (x) std::memcpy(x, it->second.x.data(), c->n * sizeof(double));
  if (iters) *iters = it->second.iters;
  c->running_or_held -= 1;
  c->reqs.erase(it);
  return SG_OK;
}

int sg_engine_cancel(sg_ctx* c, int64_t id) {
  if (!c) return SG_ERR_INVALID;
  auto it = c->reqs.find(id);
  if (it == c->reqs.end()) return fail(c, SG_ERR_NOT_FOUND, "unknown request");
  detach(c, id);
  it = c->reqs.find(id);
  if (it->second.state != Q_QUEUED) c->running_or_held -= 1;
  c->reqs.erase(it);
  return SG_OK;
}

int sg_engine_poll(sg_ctx* c, int64_t* ids, int64_t max_ids, int64_t* n_out) {
  if (!c || !n_out || (max_ids > 0 && !ids)) return SG_ERR_INVALID;
  const int64_t k = std::min<int64_t>(max_ids, (int64_t)c->finished.size());
  for (int64_t i = 0; i < k; ++i) ids[i] = c->finished[i];
  c->finished.erase(c->finished.begin(), c->finished.begin() + k);
  *n_out = k;
  return SG_OK;
}

int sg_engine_stats(sg_ctx* c, int64_t* s4) {
  if (!c || !s4) return SG_ERR_INVALID;
  s4[0] = c->steps;
  s4[1] = c->retired;
  s4[2] = c->col_iters;
  s4[3] = c->steps;
  return SG_OK;
}

int sg_engine_timing(sg_ctx* c, double* t6) {
  if (!c || !t6) return SG_ERR_INVALID;
  for (int i = 0; i < 6; ++i) t6[i] = 0.0;
  t6[0] = (double)c->steps * c->step_ms;
  return SG_OK;
}

int sg_engine_probe_cache_clear(sg_ctx* c, int64_t slot) {
  if (!c) return SG_ERR_INVALID;
  if (slot < 0) {
    for (auto& s : c->slots) s.cache.clear();
  } else if (slot < (int64_t)c->slots.size()) {
    c->slots[slot].cache.clear();
  }
  return SG_OK;
}

int sg_engine_probe_cached(sg_ctx* c, int64_t slot, uint64_t seed, int64_t run) {
  if (!c || slot < 0 || slot >= (int64_t)c->slots.size()) return 0;
  return c->slots[slot].cache.count({seed, run}) ? 1 : 0;
}

int sg_engine_probe_dots(sg_ctx* c, int64_t slot, const int64_t* ids_pcg, const int64_t* ids_prod, int64_t k,
                         uint64_t seed, int64_t run0, const double* SX, int64_t p, double* out, int32_t* iters) {
  if (!c || k <= 0 || !ids_pcg || !ids_prod || !out || p < 0 || p > 16 || (p > 0 && !SX))
    return fail(c, SG_ERR_INVALID, "probe_dots: bad arguments");
  if (slot < 0 || slot >= (int64_t)c->slots.size()) return fail(c, SG_ERR_INVALID, "bad slot");
  Slot& s = c->slots[slot];
  const int64_t n = c->n, nv = 2 + 2 * p;
  for (int64_t j = 0; j < k; ++j) {
    auto is = c->reqs.find(ids_pcg[j]);
    if (is == c->reqs.end() || is->second.state != Q_DONE) return fail(c, SG_ERR_STATE, "probe solve not finished");
    const std::vector<double>& su = is->second.x;
    std::vector<double> au;
    if (ids_prod[j] < 0) {
      auto ic = s.cache.find({seed, run0 + j});
      if (ic == s.cache.end()) return fail(c, SG_ERR_STATE, "probe product not cached");
      au = ic->second;
    } else {
      auto ia = c->reqs.find(ids_prod[j]);
      if (ia == c->reqs.end() || ia->second.state != Q_DONE) return fail(c, SG_ERR_STATE, "probe product not finished");
      au = ia->second.x;
      s.cache[{seed, run0 + j}] = au;
    }
    std::vector<double> u(n, 0.0);
    for (int64_t i = 0; i < n; ++i)
      u[i] = s.mask[i] ? ((hash3(seed, (uint64_t)(run0 + j), (uint64_t)i) >> 63) ? 1.0 : -1.0) : 0.0;
    double* row = out + j * nv;
    row[0] = dot(au, su);
    row[1] = dot(u, su);
    for (int64_t q = 0; q < p; ++q) {
      double a = 0.0, b = 0.0;
      for (int64_t i = 0; i < n; ++i) {
        a += au[i] * SX[q * n + i];
        b += SX[q * n + i] * u[i];
      }
      row[2 + q] = a;
      row[2 + p + q] = b;
    }
    if (iters) iters[j] = is->second.iters;
  }
  for (int64_t j = 0; j < 2 * k; ++j) {
    const int64_t id = j < k ? ids_pcg[j] : ids_prod[j - k];
    if (id < 0) continue;
    detach(c, id);
    c->reqs.erase(id);
    c->running_or_held -= 1;
  }
  return SG_OK;
}

}  // extern "C"
