// Native batched null-model fits.
//
// The AI-REML driver of glmmkin.ai_PCG_Rcpp_Binary / _Quantitative (FIT.R:79-304, 309-549) with
// Get_Coef (FIT.R:2-35), getCoefficients (FIT.cpp:3167-3199), getAIScore / getAIScore_q
// (FIT.cpp:3279-3295, 3479-3531), GetTrace / GetTrace_q (FIT.cpp:3113-3160, 3409-3472) and the tau
// updates of fitglmmaiRPCG / fitglmmaiRPCG_q (FIT.cpp:3302-3341, 3610-3662), run for many
// phenotypes at once.  Each fit is a state machine that issues right-hand sides to the
// continuous-batching engine and waits for them; the scheduler steps the engine (launch the next
// step, then work on the previous step's results) and resumes the fits whose columns are done.
// All vector arithmetic here is O(n p) per fit and stage, in FP64, fused into single passes.
//
// This file is a client of the engine's own C ABI (sg_engine_*): it holds no device state.
#include "host_math.h"
#include "../../include/saigegpu.h"

#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstring>
#include <functional>
#include <mutex>
#include <thread>
#include <deque>
#include <exception>
#include <map>
#include <memory>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

enum Phase { P_INIT_COEF, P_INIT_AI, P_LOOP_COEF, P_LOOP_AI, P_FINAL_COEF, P_DONE };
enum Stage { S_NONE, S_GC_WAIT, S_AI_WAIT_PROBES, S_AI_WAIT_SID };

struct FitError {
  int code;
  std::string msg;
};

struct AiScore {
  double YPAPY = 0, YPA0PY = 0, tr0 = 0, tr1 = 0;
  double AI[4] = {0, 0, 0, 0};  // column-major 2x2 (quantitative) or AI[0] (binary)
};

struct Fit {
  int64_t id = 0, slot = -1;
  bool quant = false;
  int64_t n = 0, ns = 0;
  int p = 0;
  std::vector<uint8_t> mask;  // cohort-length, 1 = in the fit's sample subset
  bool has_mask = false;
  std::vector<int64_t> idx;   // subset position -> cohort position
  // inputs over the cohort (0 outside the subset)
  std::vector<double> y, offset;
  // [Y | X]: Get_Coef's working vector, then the covariates (n x (1 + p), column-major), so that
  // Get_Coef's right-hand sides go to the engine as they are
  std::vector<double> YX;
  std::vector<double> eta, alpha;  // current eta (with offset) and coefficients of the main loop
  double tol = 0.02, tol_pcg = 1e-5, cutoff = 0.0025;
  int maxiter = 20, maxiter_pcg = 500, nrun = 30;
  uint64_t seed = 200;
  // main loop
  Phase phase = P_INIT_COEF;
  Stage stage = S_NONE;
  double tau[2] = {1.0, 0.0}, tau0[2] = {1.0, 0.0};
  std::vector<double> alpha0, eta0;
  int main_iter = 0, it_used = 0;
  // Get_Coef
  double gc_tau[2] = {0, 0};
  int gc_iter = 0;
  std::vector<double> gc_alpha0, mu, W;
  // result of the last Get_Coef
  std::vector<double> rc_alpha, rc_eta, rc_cov, SY, SX;
  // getAIScore
  std::vector<double> ai_cov, PY, APY;
  int64_t apy_id = -1;
  std::vector<int64_t> pid, aid, sid;
  int64_t run0 = 0, k = 0;
  std::vector<double> t1, t0;
  // waiting
  std::vector<int64_t> wait_ids;
  bool wait_fetch = false;
  std::vector<std::vector<double>> fetched;  // kept between stages (their buffers are reused)
  // bookkeeping
  int64_t column_iterations = 0, columns = 0;
  bool failed = false;
  FitError err;
  bool converged = false;
  int64_t ready_at = -1;  // scheduler step at which every awaited column was done
  bool started = false;   // main_start has run
  bool busy = false;      // handed to a worker thread (only the stepping thread reads or writes it)
  int64_t reserved = 0;   // engine columns set aside at admission until main_start has submitted
  double t_submit = 0, t_admit = 0, t_done = 0;  // steady-clock seconds: added, given a slot, retired
};

// Host threads that resume fits.  The thread that steps the engine hands a fit over (push) and
// takes it back once the fit waits for columns again (take_done): a fit is in the hands of one
// thread at a time.  Each worker makes the context's GPU current once (the engine calls it makes
// run under the fit driver's lock).
class Workers {
 public:
  Workers(int workers, sg_ctx* ctx, std::function<void(Fit&)> fn) : fn_(std::move(fn)) {
    for (int w = 0; w < workers; ++w)
      th_.emplace_back([this, ctx] {
        sg_ctx_make_current(ctx);
        for (;;) {
          Fit* f = nullptr;
          {
            std::unique_lock<std::mutex> lk(m_);
            cv_.wait(lk, [&] { return stop_ || !q_.empty(); });
            if (stop_) return;
            f = q_.front();
            q_.pop_front();
            ++running_;
          }
          const double t = now_s();
          fn_(*f);
          {
            std::lock_guard<std::mutex> lk(m_);
            --running_;
            busy_s_ += now_s() - t;
            done_.push_back(f);
          }
          done_cv_.notify_all();
        }
      });
  }
  // Fits still queued are dropped; call wait_idle first to keep them.
  ~Workers() {
    {
      std::lock_guard<std::mutex> lk(m_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto& t : th_) t.join();
  }
  void push(const std::vector<Fit*>& fits) {
    if (fits.empty()) return;
    {
      std::lock_guard<std::mutex> lk(m_);
      q_.insert(q_.end(), fits.begin(), fits.end());
    }
    cv_.notify_all();
  }
  // Appends the fits resumed since the last call.
  void take_done(std::vector<Fit*>& out) {
    std::lock_guard<std::mutex> lk(m_);
    out.insert(out.end(), done_.begin(), done_.end());
    done_.clear();
  }
  void wait_idle() {
    std::unique_lock<std::mutex> lk(m_);
    done_cv_.wait(lk, [&] { return q_.empty() && running_ == 0; });
  }
  // wait_idle for at most `seconds`; true if idle
  bool wait_idle_for(double seconds) {
    std::unique_lock<std::mutex> lk(m_);
    return done_cv_.wait_for(lk, std::chrono::duration<double>(seconds),
                             [&] { return q_.empty() && running_ == 0; });
  }
  double busy_seconds() {
    std::lock_guard<std::mutex> lk(m_);
    return busy_s_;
  }

 private:
  std::function<void(Fit&)> fn_;
  std::vector<std::thread> th_;
  std::mutex m_;
  std::condition_variable cv_, done_cv_;
  std::deque<Fit*> q_;
  std::vector<Fit*> done_;
  int running_ = 0;
  double busy_s_ = 0.0;
  bool stop_ = false;
};

}  // namespace

struct sg_fits {
  sg_ctx* ctx = nullptr;
  int64_t n = 0, max_columns = 0, max_fits = 0;
  // engine slots beyond max_fits: the next queued fits take them while they wait, so that their
  // subsets' set-ups (QC, tables, diagonal) run on the device before a running fit makes room
  int64_t ahead = 0;
  bool pipelined = true, launched = false;
  double t_created = 0;  // steady-clock seconds at sg_fits_create
  std::vector<int64_t> free_slots;
  std::map<int64_t, std::unique_ptr<Fit>> active;   // admitted, running
  std::deque<std::unique_ptr<Fit>> pending;          // waiting for room (the first may hold a slot)
  std::map<int64_t, std::unique_ptr<Fit>> done_fits; // finished, not yet collected
  std::deque<int64_t> finished_order;
  std::unordered_map<int64_t, int64_t> owner;        // request id -> fit id
  std::unordered_set<int64_t> done_reqs;
  int64_t next_id = 1, inflight_columns = 0;
  int64_t reserved_columns = 0;  // sum of Fit::reserved
  std::string err;
  double t_engine = 0, t_host = 0;
  double t_pheno = 0, t_submit = 0, t_fetch = 0, t_dots = 0;  // parts of t_host spent in engine calls
  double t_launch = 0;                                          // part of t_engine spent launching
  // parts of t_engine on the stepping thread with workers: waiting for the step, for the driver's
  // lock (an engine call of a worker in progress), finishing the step, scanning for ready fits
  double t_wait = 0, t_lock = 0, t_finish = 0, t_scan = 0;
  double gpu_ms_seen = 0;                                      // engine step time already budgeted
  double launch_wait_s = 0.0;  // with workers: how long a launch may wait for the fits just made ready
  int idle_passes = 0;         // consecutive stepping passes in which nothing could run
  int64_t steps = 0;
  std::mutex mu;                  // engine calls and the bookkeeping above, from the worker threads
  std::atomic<bool> step_wants{false};  // the stepping thread is waiting for mu: workers hold back
  std::unique_ptr<Workers> pool;  // null: the fits' arithmetic runs on the calling thread
};

namespace {

int fits_err(sg_fits* F, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  F->err = buf;
  return code;
}

int64_t need_columns(const Fit& f) { return 2 * (int64_t)(f.nrun + 10) + 8; }

// --------------------------------------------------------------- vector helpers (cohort length)
// binomial(logit) / gaussian working vector and weights of Get_Coef (FIT.R:4-8); R's logit
// thresholds: |eta| > 30 clamps mu.eta to DBL_EPSILON and mu to eps / (1 + eps) or its complement.
void working(Fit& f, const std::vector<double>& et) {
  const double eps = 2.220446049250313e-16;
  f.mu.resize(f.n);
  f.W.resize(f.n);
  for (int64_t i = 0; i < f.n; ++i) {
    const double e = et[i];
    double mu, mu_eta, var;
    if (f.quant) {
      mu = e;
      mu_eta = 1.0;
      var = 1.0;
    } else {
      const double ex = std::exp(std::min(std::max(e, -30.0), 30.0));
      const double tmp = e < -30.0 ? eps : (e > 30.0 ? 1.0 / eps : ex);
      mu = tmp / (1.0 + tmp);
      mu_eta = (e > 30.0 || e < -30.0) ? eps : ex / ((1.0 + ex) * (1.0 + ex));
      var = mu * (1.0 - mu);
    }
    f.mu[i] = mu;
    const bool in = f.mask[i] != 0;
    f.YX[i] = in ? e - f.offset[i] + (f.y[i] - mu) / mu_eta : 0.0;
    if (f.quant) {
      f.W[i] = 1.0;
    } else {
      const double r = mu_eta / std::sqrt(var);
      f.W[i] = in ? r * r : 1.0;
    }
  }
}

// A' B for column-major n x a and n x b.  Every entry is summed in row order, as one dot product
// at a time would sum it, but the entries advance together in one pass over the rows: the loop is
// bound by throughput instead of by the latency of a single chain of additions (sizes up to 8 x 8
// get their accumulators in registers).
template <int NA, int NB>
void gram_fixed(const double* A, const double* B, int64_t n, double* out) {
  double acc[NA * NB] = {};
  for (int64_t r = 0; r < n; ++r) {
    double x[NA];
    for (int i = 0; i < NA; ++i) x[i] = A[(int64_t)i * n + r];
    for (int j = 0; j < NB; ++j) {
      const double z = B[(int64_t)j * n + r];
      for (int i = 0; i < NA; ++i) acc[i + j * NA] += x[i] * z;
    }
  }
  for (int k = 0; k < NA * NB; ++k) out[k] = acc[k];
}

template <int NA>
bool gram_dispatch_b(const double* A, const double* B, int b, int64_t n, double* out) {
  if (b == 1) gram_fixed<NA, 1>(A, B, n, out);
  else if (b == NA) gram_fixed<NA, NA>(A, B, n, out);
  else return false;
  return true;
}

void gram(const double* A, int a, const double* B, int b, int64_t n, double* out) {
  bool done = false;
  switch (a) {
    case 1: done = gram_dispatch_b<1>(A, B, b, n, out); break;
    case 2: done = gram_dispatch_b<2>(A, B, b, n, out); break;
    case 3: done = gram_dispatch_b<3>(A, B, b, n, out); break;
    case 4: done = gram_dispatch_b<4>(A, B, b, n, out); break;
    case 5: done = gram_dispatch_b<5>(A, B, b, n, out); break;
    case 6: done = gram_dispatch_b<6>(A, B, b, n, out); break;
    case 7: done = gram_dispatch_b<7>(A, B, b, n, out); break;
    case 8: done = gram_dispatch_b<8>(A, B, b, n, out); break;
    default: break;
  }
  if (done) return;
  std::vector<double> acc((size_t)a * b, 0.0);
  for (int64_t r = 0; r < n; ++r)
    for (int j = 0; j < b; ++j) {
      const double z = B[(int64_t)j * n + r];
      for (int i = 0; i < a; ++i) acc[i + j * a] += A[(int64_t)i * n + r] * z;
    }
  std::copy(acc.begin(), acc.end(), out);
}

// k dot products a_q . b_q of length n in one pass (each summed in index order)
template <int K>
void dots(const double* const* a, const double* const* b, int64_t n, double* out) {
  double acc[K] = {};
  for (int64_t i = 0; i < n; ++i)
    for (int q = 0; q < K; ++q) acc[q] += a[q][i] * b[q][i];
  for (int q = 0; q < K; ++q) out[q] = acc[q];
}

// out = v - SX (cov (SX' w)): the projection P applied as the reference writes it
void project(const Fit& f, const std::vector<double>& cov, const double* v, const double* w, double* out) {
  const int p = f.p;
  std::vector<double> a(p), b(p, 0.0);
  gram(f.SX.data(), p, w, 1, f.n, a.data());
  for (int i = 0; i < p; ++i)
    for (int j = 0; j < p; ++j) b[i] += cov[i + j * p] * a[j];
  for (int64_t r = 0; r < f.n; ++r) {
    double s = 0.0;
    for (int j = 0; j < p; ++j) s += f.SX[r + (int64_t)j * f.n] * b[j];
    out[r] = v[r] - s;
  }
}

double cal_cv(const std::vector<double>& x) {
  const double nn = (double)x.size();
  double m = 0.0;
  for (double v : x) m += v;
  m /= nn;
  double ss = 0.0;
  for (double v : x) ss += (v - m) * (v - m);
  const double sd = std::sqrt(ss / (nn - 1.0));
  return (sd / m) / nn;
}

// --------------------------------------------------------------- engine requests
void fail(sg_fits* F, Fit& f, int code, const std::string& msg) {
  if (!f.failed) {
    f.failed = true;
    f.err = FitError{code, msg};
  }
}

// The driver's lock as a worker takes it: after the stepping thread, which is waiting to turn a
// finished step around (StepLock), so that it waits for at most the engine call in progress.
std::unique_lock<std::mutex> worker_lock(sg_fits* F) {
  while (F->step_wants.load(std::memory_order_acquire)) std::this_thread::yield();
  return std::unique_lock<std::mutex>(F->mu);
}

struct StepLock {
  sg_fits* F;
  explicit StepLock(sg_fits* f) : F(f) {
    F->step_wants.store(true, std::memory_order_release);
    F->mu.lock();
    F->step_wants.store(false, std::memory_order_release);
  }
  ~StepLock() { F->mu.unlock(); }
};

// One engine call (and whatever bookkeeping fn does with its result) under the fit driver's lock.
template <typename Fn>
bool eng(sg_fits* F, Fit& f, double* timer, Fn fn) {
  const auto g = worker_lock(F);
  const double t = now_s();
  const int rc = fn();
  if (timer) *timer += now_s() - t;
  if (rc == SG_OK) return true;
  const char* m = sg_last_error(F->ctx);
  fail(F, f, rc, m ? m : "engine error");
  return false;
}

void own(sg_fits* F, Fit& f, const std::vector<int64_t>& ids) {
  for (int64_t id : ids)
    if (id >= 0) F->owner[id] = f.id;
  f.columns += (int64_t)ids.size();
  F->inflight_columns += (int64_t)ids.size();
}

bool set_pheno(sg_fits* F, Fit& f, const std::vector<double>& W, const double* tau) {
  const uint8_t* mask = f.has_mask ? f.mask.data() : nullptr;
  // a new subset: its QC and tables run on the device while this thread waits without the lock,
  // so the stepping thread can turn steps around meanwhile (no-ops once the slot holds the subset)
  if (!eng(F, f, &F->t_pheno, [&] { return sg_engine_prepare_subset(F->ctx, f.slot, mask); })) return false;
  const double t = now_s();
  sg_engine_subset_wait(F->ctx, f.slot);
  {
    std::lock_guard<std::mutex> g(F->mu);
    F->t_pheno += now_s() - t;
  }
  return eng(F, f, &F->t_pheno, [&] { return sg_engine_set_pheno(F->ctx, f.slot, W.data(), tau, mask); });
}

bool submit(sg_fits* F, Fit& f, int kind, const double* B, int64_t k, int maxiter, double tol,
            std::vector<int64_t>& ids) {
  ids.assign(k, -1);
  return eng(F, f, &F->t_submit, [&] {
    const int rc = sg_engine_submit(F->ctx, f.slot, kind, B, k, maxiter, tol, ids.data());
    if (rc == SG_OK) own(F, f, ids);
    return rc;
  });
}

// one PCG solve of Sigma x = (result of request src), chained on the engine
bool submit_chained(sg_fits* F, Fit& f, int64_t src, std::vector<int64_t>& ids) {
  ids.assign(1, -1);
  return eng(F, f, &F->t_submit, [&] {
    const int rc = sg_engine_submit_chained(F->ctx, f.slot, &src, 1, f.maxiter_pcg, f.tol_pcg, ids.data());
    if (rc == SG_OK) own(F, f, ids);
    return rc;
  });
}

bool submit_probes(sg_fits* F, Fit& f, int64_t run0, int64_t k, std::vector<int64_t>& ids) {
  ids.assign(k, -1);
  return eng(F, f, &F->t_submit, [&] {
    const int rc = sg_engine_submit_probes(F->ctx, f.slot, 0, f.seed, run0, k, f.maxiter_pcg, f.tol_pcg, ids.data());
    if (rc == SG_OK) own(F, f, ids);
    return rc;
  });
}

// K u of the probes: -1 where the slot's cache holds it (same probes and sample mask all fit
// long), else maximal runs of uncached probes submitted as product blocks
bool probe_products(sg_fits* F, Fit& f, int64_t run0, int64_t cnt, std::vector<int64_t>& out) {
  out.assign(cnt, -1);
  return eng(F, f, &F->t_submit, [&] {
    int64_t j = 0;
    while (j < cnt) {
      if (sg_engine_probe_cached(F->ctx, f.slot, f.seed, run0 + j)) {
        ++j;
        continue;
      }
      int64_t j1 = j;
      while (j1 < cnt && !sg_engine_probe_cached(F->ctx, f.slot, f.seed, run0 + j1)) ++j1;
      std::vector<int64_t> ids(j1 - j, -1);
      const int rc = sg_engine_submit_probes(F->ctx, f.slot, 1, f.seed, run0 + j, j1 - j, 1, 0.0, ids.data());
      if (rc != SG_OK) return rc;
      own(F, f, ids);
      for (int64_t q = 0; q < j1 - j; ++q) out[j + q] = ids[q];
      j = j1;
    }
    return (int)SG_OK;
  });
}

void wait_for(Fit& f, Stage st, std::vector<int64_t> ids, bool fetch) {
  f.stage = st;
  f.wait_ids.clear();
  for (int64_t id : ids)
    if (id >= 0) f.wait_ids.push_back(id);
  f.wait_fetch = fetch;
}

// --------------------------------------------------------------- Get_Coef
bool gc_issue(sg_fits* F, Fit& f) {
  if (!set_pheno(F, f, f.W, f.gc_tau)) return false;
  std::vector<int64_t> ids;
  if (!submit(F, f, 0, f.YX.data(), 1 + f.p, f.maxiter_pcg, f.tol_pcg, ids)) return false;
  wait_for(f, S_GC_WAIT, ids, true);
  return true;
}

bool gc_begin(sg_fits* F, Fit& f, const double* tau, const std::vector<double>& alpha0,
              const std::vector<double>& eta0) {
  f.gc_tau[0] = tau[0];
  f.gc_tau[1] = tau[1];
  f.gc_alpha0 = alpha0;
  f.gc_iter = 0;
  working(f, eta0);
  return gc_issue(F, f);
}

// getCoefficients on the solved [Sigma^-1 Y, Sigma^-1 X] (Sigma^-1 X fetched into SX by resume);
// returns true when Get_Coef is done
bool gc_step(sg_fits* F, Fit& f, bool* done) {
  const int p = f.p;
  const int64_t n = f.n;
  f.SY.swap(f.fetched[0]);
  std::vector<double> XtSX(p * p);
  gram(f.YX.data() + n, p, f.SX.data(), p, n, XtSX.data());
  f.rc_cov = sg::inv_sympd(XtSX, p);
  std::vector<double> sxy(p);
  gram(f.SX.data(), p, f.YX.data(), 1, n, sxy.data());
  std::vector<double> al(p, 0.0);
  for (int i = 0; i < p; ++i)
    for (int j = 0; j < p; ++j) al[i] += f.rc_cov[i + j * p] * sxy[j];
  std::vector<double> et(n);
  for (int64_t r = 0; r < n; ++r) {
    double s = 0.0;
    for (int j = 0; j < p; ++j) s += f.SX[r + (int64_t)j * n] * al[j];
    et[r] = (f.mask[r] ? f.YX[r] - f.gc_tau[0] * (f.SY[r] - s) / f.W[r] : 0.0) + f.offset[r];
  }
  working(f, et);
  ++f.gc_iter;
  double dmax = 0.0;
  for (int i = 0; i < p; ++i)
    dmax = std::max(dmax, std::fabs(al[i] - f.gc_alpha0[i]) / (std::fabs(al[i]) + std::fabs(f.gc_alpha0[i]) + 0.1));
  f.rc_alpha = al;
  f.rc_eta = et;
  if (dmax < 0.1 || f.gc_iter >= f.maxiter) {
    *done = true;
    return true;
  }
  f.gc_alpha0 = al;
  *done = false;
  return gc_issue(F, f);
}

// --------------------------------------------------------------- getAIScore
bool ai_begin(sg_fits* F, Fit& f) {
  const int p = f.p;
  const int64_t n = f.n;
  if (!set_pheno(F, f, f.W, f.tau)) return false;
  if (f.quant) {
    std::vector<double> XtSX(p * p);
    gram(f.YX.data() + n, p, f.SX.data(), p, n, XtSX.data());
    f.ai_cov = sg::inv_sympd(XtSX, p);
  } else {
    f.ai_cov = f.rc_cov;
  }
  f.PY.resize(n);
  project(f, f.ai_cov, f.SY.data(), f.YX.data(), f.PY.data());
  // APY = K PY, then Sigma^-1 APY chained to it on the engine (admitted as soon as the product is
  // done, no trip through the host) and, quantitative, Sigma^-1 PY; APY itself is fetched with them
  std::vector<int64_t> a;
  if (!submit(F, f, 1, f.PY.data(), 1, 1, 0.0, a)) return false;
  f.apy_id = a[0];
  if (!submit_chained(F, f, f.apy_id, f.sid)) return false;
  if (f.quant) {
    std::vector<int64_t> q;
    if (!submit(F, f, 0, f.PY.data(), 1, f.maxiter_pcg, f.tol_pcg, q)) return false;
    f.sid.push_back(q[0]);
  }
  if (!submit_probes(F, f, 0, f.nrun, f.pid)) return false;
  if (!probe_products(F, f, 0, f.nrun, f.aid)) return false;
  f.run0 = 0;
  f.k = f.nrun;
  f.t1.clear();
  f.t0.clear();
  std::vector<int64_t> w(f.pid);
  w.insert(w.end(), f.aid.begin(), f.aid.end());
  wait_for(f, S_AI_WAIT_PROBES, w, false);
  return true;
}

bool ai_after_probes(sg_fits* F, Fit& f) {
  const int p = f.p;
  const int64_t nv = 2 + 2 * p, k = (int64_t)f.pid.size();
  std::vector<double> D(k * nv);
  std::vector<int32_t> its(k, 0);
  // launch the reduction, wait for it without the lock (the stepping thread may turn a step
  // around meanwhile), then collect it
  if (!eng(F, f, &F->t_dots, [&] {
        return sg_engine_probe_dots_begin(F->ctx, f.slot, f.pid.data(), f.aid.data(), k, f.seed, f.run0,
                                          f.SX.data(), p);
      }))
    return false;
  const double tw = now_s();
  sg_engine_probe_dots_wait(F->ctx, f.slot);
  {
    std::lock_guard<std::mutex> g(F->mu);
    F->t_dots += now_s() - tw;
  }
  const bool ok = eng(F, f, &F->t_dots, [&] {
    const int rc = sg_engine_probe_dots_end(F->ctx, f.slot, D.data(), its.data());
    if (rc != SG_OK) return rc;
    for (int64_t j = 0; j < k; ++j) {
      F->done_reqs.erase(f.pid[j]);
      F->owner.erase(f.pid[j]);
      if (f.aid[j] >= 0) {
        F->done_reqs.erase(f.aid[j]);
        F->owner.erase(f.aid[j]);
      }
    }
    return rc;
  });
  if (!ok) return false;
  for (int64_t j = 0; j < k; ++j) f.column_iterations += its[j] + (f.aid[j] >= 0 ? 1 : 0);
  for (int64_t j = 0; j < k; ++j) {
    const double* row = D.data() + j * nv;
    const double* b = row + 2;
    const double* c = row + 2 + p;
    double bcc = 0.0, ccc = 0.0;
    for (int i = 0; i < p; ++i)
      for (int q = 0; q < p; ++q) {
        bcc += b[i] * f.ai_cov[i + q * p] * c[q];
        ccc += c[i] * f.ai_cov[i + q * p] * c[q];
      }
    f.t1.push_back(row[0] - bcc);
    f.t0.push_back(row[1] - ccc);
  }
  if (cal_cv(f.t1) > f.cutoff || (f.quant && cal_cv(f.t0) > f.cutoff)) {
    f.run0 += f.k;
    f.k = 10;
    if (!submit_probes(F, f, f.run0, f.k, f.pid)) return false;
    if (!probe_products(F, f, f.run0, f.k, f.aid)) return false;
    std::vector<int64_t> w(f.pid);
    w.insert(w.end(), f.aid.begin(), f.aid.end());
    wait_for(f, S_AI_WAIT_PROBES, w, false);
    return true;
  }
  std::vector<int64_t> w{f.apy_id};
  w.insert(w.end(), f.sid.begin(), f.sid.end());
  wait_for(f, S_AI_WAIT_SID, w, true);
  return true;
}

AiScore ai_finish(Fit& f) {
  const int64_t n = f.n;
  AiScore re;
  std::vector<double> PAPY(n);
  f.APY.swap(f.fetched[0]);
  project(f, f.ai_cov, f.fetched[1].data(), f.fetched[1].data(), PAPY.data());
  double s1 = 0.0, s0 = 0.0;
  for (double v : f.t1) s1 += v;
  for (double v : f.t0) s0 += v;
  re.tr1 = s1 / (double)f.t1.size();
  re.tr0 = s0 / (double)f.t0.size();
  const double* py = f.PY.data();
  const double* apy = f.APY.data();
  if (f.quant) {
    std::vector<double> PA0PY(n);
    project(f, f.ai_cov, f.fetched[2].data(), f.fetched[2].data(), PA0PY.data());
    const double* a[5] = {py, py, py, py, apy};
    const double* b[5] = {apy, py, PA0PY.data(), PAPY.data(), PAPY.data()};
    double d[5];
    dots<5>(a, b, n, d);
    re.YPAPY = d[0];
    re.YPA0PY = d[1];
    re.AI[0] = d[2];
    re.AI[1] = re.AI[2] = d[3];
    re.AI[3] = d[4];
  } else {
    const double* a[2] = {py, apy};
    const double* b[2] = {apy, PAPY.data()};
    double d[2];
    dots<2>(a, b, n, d);
    re.YPAPY = d[0];
    re.AI[0] = d[1];
  }
  return re;
}

// --------------------------------------------------------------- tau updates
void tau_update(Fit& f, const AiScore& re) {
  const double tol = f.tol;
  const double t0[2] = {f.tau[0], f.tau[1]};
  if (!f.quant) {  // fitglmmaiRPCG
    const double dtau = (re.YPAPY - re.tr1) / re.AI[0];
    double t[2] = {t0[0], t0[1] + dtau};
    for (double& v : t)
      if (v < tol) v = 0.0;
    double step = 1.0;
    while (t[1] < 0.0) {
      step *= 0.5;
      t[1] = t0[1] + step * dtau;
    }
    for (double& v : t)
      if (v < tol) v = 0.0;
    f.tau[0] = t[0];
    f.tau[1] = t[1];
    return;
  }
  // fitglmmaiRPCG_q: dtau = AI^-1 score (2 x 2, partial pivoting)
  const bool zero[2] = {t0[0] < tol, t0[1] < tol};
  const double sc[2] = {re.YPA0PY - re.tr0, re.YPAPY - re.tr1};
  double a = re.AI[0], b = re.AI[2], c = re.AI[1], d = re.AI[3];  // [[a b] [c d]]
  double r0 = sc[0], r1 = sc[1];
  double dt[2];
  if (std::fabs(c) > std::fabs(a)) {
    std::swap(a, c);
    std::swap(b, d);
    std::swap(r0, r1);
  }
  const double l = c / a;
  const double d2 = d - l * b, r2 = r1 - l * r0;
  dt[1] = r2 / d2;
  dt[0] = (r0 - b * dt[1]) / a;
  double t[2] = {t0[0] + dt[0], t0[1] + dt[1]};
  for (int i = 0; i < 2; ++i)
    if (zero[i] && t[i] < tol) t[i] = 0.0;
  double step = 1.0;
  while (t[0] < 0.0 || t[1] < 0.0) {
    step *= 0.5;
    for (int i = 0; i < 2; ++i) {
      t[i] = t0[i] + step * dt[i];
      if (zero[i] && t[i] < tol) t[i] = 0.0;
    }
  }
  for (double& v : t)
    if (v < tol) v = 0.0;
  f.tau[0] = t[0];
  f.tau[1] = t[1];
}

// --------------------------------------------------------------- main loop (glmmkin.ai_PCG_Rcpp_*)
bool main_start(sg_fits* F, Fit& f) {
  f.alpha0 = f.alpha;
  f.eta0 = f.eta;
  if (f.quant) {
    working(f, f.eta);
    double m = 0.0;
    for (int64_t i : f.idx) m += f.YX[i];
    m /= (double)f.ns;
    double ss = 0.0;
    for (int64_t i : f.idx) ss += (f.YX[i] - m) * (f.YX[i] - m);
    if (std::fabs(ss / (double)(f.ns - 1)) < 0.1) {
      fail(F, f, SG_ERR_NUMERIC, "variance of the phenotype is much smaller than 1");
      return false;
    }
    f.tau[0] = 1.0;
    f.tau[1] = 0.0;
  } else {
    f.tau[0] = 1.0;
    f.tau[1] = 0.1;
  }
  f.tau0[0] = f.tau[0];
  f.tau0[1] = f.tau[1];
  f.phase = P_INIT_COEF;
  return gc_begin(F, f, f.tau, f.alpha0, f.eta0);
}

bool final_coef(sg_fits* F, Fit& f) {
  f.phase = P_FINAL_COEF;
  return gc_begin(F, f, f.tau, f.alpha, f.eta);
}

bool loop_next(sg_fits* F, Fit& f) {
  if (f.main_iter >= f.maxiter) return final_coef(F, f);
  f.main_iter += 1;
  f.it_used = f.main_iter;
  f.alpha0 = f.quant ? f.alpha : f.rc_alpha;
  f.tau0[0] = f.tau[0];
  f.tau0[1] = f.tau[1];
  f.eta0 = f.eta;
  f.phase = P_LOOP_COEF;
  return gc_begin(F, f, f.tau, f.alpha0, f.eta0);
}

bool coef_done(sg_fits* F, Fit& f) {
  switch (f.phase) {
    case P_INIT_COEF:
      f.phase = P_INIT_AI;
      return ai_begin(F, f);
    case P_LOOP_COEF:
      f.phase = P_LOOP_AI;
      return ai_begin(F, f);
    case P_FINAL_COEF:
      f.phase = P_DONE;
      f.stage = S_NONE;
      f.converged = f.it_used < f.maxiter;
      return true;
    default:
      fail(F, f, SG_ERR_STATE, "fit state machine: Get_Coef finished in an unexpected phase");
      return false;
  }
}

bool ai_done(sg_fits* F, Fit& f, const AiScore& re) {
  const double n = (double)f.ns;
  if (f.phase == P_INIT_AI) {  // the first, damped step (FIT.R:165, 405-406)
    if (f.quant) {
      f.tau[1] = std::max(0.0, f.tau0[1] + f.tau0[1] * f.tau0[1] * (re.YPAPY - re.tr1) / n);
      f.tau[0] = std::max(0.0, f.tau0[0] + f.tau0[0] * f.tau0[0] * (re.YPA0PY - re.tr0) / n);
    } else {
      f.tau[1] = std::max(0.0, f.tau0[1] + f.tau0[1] * f.tau0[1] * (re.YPAPY - re.tr1) / n);
    }
    f.main_iter = 0;
    f.it_used = 0;
    return loop_next(F, f);
  }
  if (f.phase != P_LOOP_AI) {
    fail(F, f, SG_ERR_STATE, "fit state machine: AI score finished in an unexpected phase");
    return false;
  }
  tau_update(f, re);
  f.alpha = f.rc_alpha;
  f.eta = f.rc_eta;
  if (f.quant && f.tau[0] <= 0.0) {
    fail(F, f, SG_ERR_NUMERIC, "the first variance component parameter estimate is 0");
    return false;
  }
  if (f.quant ? f.tau[1] <= 0.0 : f.tau[1] == 0.0) return final_coef(F, f);
  double rel = 0.0;
  for (int i = 0; i < 2; ++i)
    rel = std::max(rel, std::fabs(f.tau[i] - f.tau0[i]) / (std::fabs(f.tau[i]) + std::fabs(f.tau0[i]) + f.tol));
  if (rel < f.tol) return final_coef(F, f);
  if (std::max(f.tau[0], f.tau[1]) > 1.0 / (f.tol * f.tol)) {
    f.it_used = f.maxiter;
    return final_coef(F, f);
  }
  return loop_next(F, f);
}

// Resume a fit whose awaited columns are done: fetch them if asked (Get_Coef's Sigma^-1 X straight
// into SX, the others into the fit's reused buffers), then run its next stage.
bool resume(sg_fits* F, Fit& f) {
  if (f.wait_fetch) {
    const size_t nw = f.wait_ids.size();
    const bool gc = f.stage == S_GC_WAIT;
    if (f.fetched.size() < nw) f.fetched.resize(nw);
    if (gc) f.SX.resize((size_t)f.n * f.p);
    for (size_t q = 0; q < nw; ++q) {
      const int64_t id = f.wait_ids[q];
      double* x;
      if (gc && q > 0) {
        x = f.SX.data() + (q - 1) * (size_t)f.n;
      } else {
        f.fetched[q].resize(f.n);
        x = f.fetched[q].data();
      }
      int32_t it = 0;
      const bool ok = eng(F, f, &F->t_fetch, [&] {
        const int rc = sg_engine_fetch(F->ctx, id, x, &it);
        if (rc == SG_OK) {
          F->done_reqs.erase(id);
          F->owner.erase(id);
        }
        return rc;
      });
      if (!ok) return false;
      f.column_iterations += it;
    }
  }
  const Stage st = f.stage;
  f.stage = S_NONE;
  f.wait_ids.clear();
  switch (st) {
    case S_GC_WAIT: {
      bool done = false;
      if (!gc_step(F, f, &done)) return false;
      return done ? coef_done(F, f) : true;
    }
    case S_AI_WAIT_PROBES:
      return ai_after_probes(F, f);
    case S_AI_WAIT_SID:
      return ai_done(F, f, ai_finish(f));
    default:
      fail(F, f, SG_ERR_STATE, "fit state machine: resumed without a pending wait");
      return false;
  }
}

// Every awaited column is done (the caller holds F->mu).
bool ready_locked(sg_fits* F, const Fit& f) {
  if (f.stage == S_NONE) return false;
  for (int64_t id : f.wait_ids)
    if (!F->done_reqs.count(id)) return false;
  return true;
}

bool is_ready(sg_fits* F, const Fit& f) {
  if (f.stage == S_NONE) return false;
  const auto g = worker_lock(F);
  return ready_locked(F, f);
}

// Start the fit if it has not started, then resume it until it waits for columns still running
// (or finishes, or fails).  On a worker thread or the calling thread; the fit is this thread's.
void advance(sg_fits* F, Fit& f) {
  try {
    if (!f.started) {
      f.started = true;
      if (!main_start(F, f) || f.failed || f.phase == P_DONE) return;
    }
    while (is_ready(F, f)) {
      f.ready_at = -1;
      if (!resume(F, f) || f.failed || f.phase == P_DONE) break;
    }
  } catch (const std::exception& ex) {
    fail(F, f, SG_ERR_NOMEM, std::string("fit driver: ") + ex.what());
  }
}

// A finished or failed fit: cancel its outstanding requests, free its slot, queue it for polling.
void retire(sg_fits* F, int64_t fid) {
  auto it = F->active.find(fid);
  if (it == F->active.end()) return;
  std::unique_ptr<Fit> f = std::move(it->second);
  F->active.erase(it);
  {
    std::lock_guard<std::mutex> g(F->mu);
    std::vector<int64_t> mine;
    for (const auto& kv : F->owner)
      if (kv.second == fid) mine.push_back(kv.first);
    for (int64_t id : mine) {
      sg_engine_cancel(F->ctx, id);
      F->owner.erase(id);
      if (!F->done_reqs.erase(id)) F->inflight_columns -= 1;
    }
  }
  F->reserved_columns -= f->reserved;
  f->reserved = 0;
  F->free_slots.push_back(f->slot);
  F->finished_order.push_back(fid);
  f->t_done = now_s();
  F->done_fits[fid] = std::move(f);
}

// Retire the fits no worker holds that finished or failed; returns how many.
int64_t retire_finished(sg_fits* F) {
  std::vector<int64_t> out;
  for (const auto& kv : F->active) {
    const Fit& f = *kv.second;
    if (!f.busy && (f.failed || f.phase == P_DONE)) out.push_back(kv.first);
  }
  for (int64_t fid : out) retire(F, fid);
  return (int64_t)out.size();
}

// Take back the fits the workers are done with.
void take_back(sg_fits* F) {
  if (!F->pool) return;
  std::vector<Fit*> back;
  F->pool->take_done(back);
  for (Fit* f : back) {
    f->busy = false;
    F->reserved_columns -= f->reserved;
    f->reserved = 0;
  }
}

// Give a queued fit a free slot: the slot's cached probe products go (a new sample mask takes it).
void take_slot(sg_fits* F, Fit& f) {
  f.slot = F->free_slots.back();
  F->free_slots.pop_back();
  std::lock_guard<std::mutex> g(F->mu);
  sg_engine_probe_cache_clear(F->ctx, f.slot);
}

// The first F->ahead queued fits hold slots while they wait, and their subsets' set-ups are
// launched there (sg_engine_prepare_subset: nothing waits for them; a failure shows again when the
// fit sets its phenotype).
void prepare_ahead(sg_fits* F) {
  int64_t k = 0;
  for (auto& p : F->pending) {
    if (k++ >= F->ahead) break;
    if (p->slot >= 0) continue;
    if (F->free_slots.empty()) break;
    take_slot(F, *p);
    std::lock_guard<std::mutex> g(F->mu);
    (void)sg_engine_prepare_subset(F->ctx, p->slot, p->has_mask ? p->mask.data() : nullptr);
  }
}

// Admit queued fits while room for max_fits fits and engine columns last.  With workers the fits
// start there (their columns are reserved until they have submitted); without, here.
void admit(sg_fits* F) {
  std::vector<Fit*> starts;
  while (!F->pending.empty() && (int64_t)F->active.size() < F->max_fits) {
    if (F->pending.front()->slot < 0 && F->free_slots.empty()) break;
    int64_t inflight;
    {
      std::lock_guard<std::mutex> g(F->mu);
      inflight = F->inflight_columns;
    }
    if (inflight + F->reserved_columns + need_columns(*F->pending.front()) > F->max_columns) break;
    std::unique_ptr<Fit> f = std::move(F->pending.front());
    F->pending.pop_front();
    if (f->slot < 0) take_slot(F, *f);
    f->t_admit = now_s();
    const int64_t fid = f->id;
    Fit& ref = *f;
    F->active[fid] = std::move(f);
    if (F->pool) {
      ref.reserved = need_columns(ref);
      F->reserved_columns += ref.reserved;
      ref.busy = true;
      starts.push_back(&ref);
      continue;
    }
    const double t = now_s();
    advance(F, ref);
    F->t_host += now_s() - t;
    if (ref.failed || ref.phase == P_DONE) retire(F, fid);
  }
  if (F->pool) F->pool->push(starts);
  prepare_ahead(F);
}

// Mark the requests the engine finished as done (the caller holds F->mu or runs alone).
int poll_done(sg_fits* F) {
  int64_t ids[1024];
  int64_t got = 0;
  do {
    const int rc = sg_engine_poll(F->ctx, ids, 1024, &got);
    if (rc != SG_OK) return rc;
    for (int64_t q = 0; q < got; ++q) {
      if (!F->owner.count(ids[q])) continue;
      if (F->done_reqs.insert(ids[q]).second) F->inflight_columns -= 1;
    }
  } while (got == 1024);
  return SG_OK;
}

}  // namespace

// ------------------------------------------------------------------ C ABI
extern "C" int sg_fits_create(sg_ctx* ctx, int64_t max_columns, int64_t max_fits, int pipelined, sg_fits** out) {
  if (!ctx || !out || max_fits <= 0 || max_columns <= 0) return SG_ERR_INVALID;
  int64_t n = 0, mt = 0, mq = 0, mv = 0;
  int rc = sg_geno_dims(ctx, &n, &mt, &mq, &mv);
  if (rc != SG_OK) return rc;
  const int64_t ahead = std::min<int64_t>(8, (max_fits + 7) / 8);
  rc = sg_engine_reserve(ctx, max_columns, max_fits + ahead);
  if (rc != SG_OK) return rc;
  rc = sg_engine_hold_results(ctx, 1);  // probe results are reduced on the device, not copied
  if (rc != SG_OK) return rc;
  sg_fits* F = new sg_fits();
  F->ctx = ctx;
  F->n = n;
  F->max_columns = max_columns;
  F->max_fits = max_fits;
  F->ahead = ahead;
  F->pipelined = pipelined != 0;
  F->t_created = now_s();
  for (int64_t s = max_fits + ahead - 1; s >= 0; --s) F->free_slots.push_back(s);
  const unsigned hw = std::thread::hardware_concurrency();
  const int workers = (int)std::min<unsigned>(7u, hw > 2 ? hw / 2 - 1 : 0u);
  if (workers > 0) F->pool.reset(new Workers(workers, ctx, [F](Fit& f) { advance(F, f); }));
  *out = F;
  return SG_OK;
}

extern "C" int sg_fits_set_threads(sg_fits* F, int threads) {
  if (!F || threads < 1) return SG_ERR_INVALID;
  if (F->pool) {  // let the current workers finish what they hold
    F->pool->wait_idle();
    take_back(F);
    F->t_host += F->pool->busy_seconds();
  }
  F->pool.reset(threads > 1 ? new Workers(threads - 1, F->ctx, [F](Fit& f) { advance(F, f); }) : nullptr);
  return SG_OK;
}

extern "C" int sg_fits_set_launch_wait(sg_fits* F, double ms) {
  if (!F || !(ms >= 0.0) || ms > 1000.0) return SG_ERR_INVALID;
  F->launch_wait_s = ms * 1e-3;
  return SG_OK;
}

extern "C" void sg_fits_destroy(sg_fits* F) {
  if (!F) return;
  if (F->pool) {
    F->pool->wait_idle();
    F->pool.reset();
  }
  if (F->launched) {
    int64_t fin = 0;
    sg_engine_finish(F->ctx, &fin);
  }
  for (const auto& kv : F->owner) sg_engine_cancel(F->ctx, kv.first);
  sg_engine_hold_results(F->ctx, 0);
  delete F;
}

extern "C" const char* sg_fits_last_error(sg_fits* F) { return F ? F->err.c_str() : "null handle"; }

static int fits_submit_impl(sg_fits* F, int trait, int64_t n_sub, const uint8_t* mask, const double* y,
                              const double* X, int p, const double* offset, const double* eta0,
                              const double* alpha0, double tol, int maxiter, int nrun, double tol_pcg,
                              int maxiter_pcg, double cv_cutoff, uint64_t seed, int64_t* fit_id) {
  if (!F) return SG_ERR_INVALID;
  if (!y || !X || !eta0 || !alpha0 || p <= 0 || n_sub <= 1 || nrun < 2 || maxiter < 1 || (trait != 0 && trait != 1))
    return fits_err(F, SG_ERR_INVALID, "sg_fits_submit: invalid arguments");
  auto f = std::make_unique<Fit>();
  f->n = F->n;
  f->quant = trait == 1;
  f->p = p;
  f->mask.assign(F->n, 1);
  f->has_mask = mask != nullptr;
  if (mask)
    for (int64_t i = 0; i < F->n; ++i) f->mask[i] = mask[i] ? 1 : 0;
  for (int64_t i = 0; i < F->n; ++i)
    if (f->mask[i]) f->idx.push_back(i);
  if ((int64_t)f->idx.size() != n_sub)
    return fits_err(F, SG_ERR_INVALID, "sg_fits_submit: n_sub = %lld but the mask selects %lld samples",
                    (long long)n_sub, (long long)f->idx.size());
  f->ns = n_sub;
  const int64_t n = F->n;
  f->y.assign(n, 0.0);
  f->YX.assign((size_t)n * (1 + p), 0.0);
  f->offset.assign(n, 0.0);
  f->eta.assign(n, 0.0);
  for (int64_t s = 0; s < n_sub; ++s) {
    const int64_t i = f->idx[s];
    f->y[i] = y[s];
    for (int j = 0; j < p; ++j) f->YX[(int64_t)(1 + j) * n + i] = X[s + (int64_t)j * n_sub];
    f->offset[i] = offset ? offset[s] : 0.0;
    f->eta[i] = eta0[s];
  }
  f->alpha.assign(alpha0, alpha0 + p);
  f->tol = tol;
  f->maxiter = maxiter;
  f->nrun = nrun;
  f->tol_pcg = tol_pcg;
  f->maxiter_pcg = maxiter_pcg;
  f->cutoff = cv_cutoff;
  f->seed = seed;
  if (need_columns(*f) > F->max_columns)
    return fits_err(F, SG_ERR_INVALID, "a fit with %d probes needs %lld engine columns, the engine has %lld", nrun,
                    (long long)need_columns(*f), (long long)F->max_columns);
  f->id = F->next_id++;
  f->t_submit = now_s();
  if (fit_id) *fit_id = f->id;
  F->pending.push_back(std::move(f));
  admit(F);
  return SG_OK;
}

// Launch the next engine step (the caller holds F->mu).
static int launch_step(sg_fits* F) {
  const double t = now_s();
  int64_t fin = 0;
  int launched = 0;
  const int rc = sg_engine_launch(F->ctx, &fin, &launched);
  F->launched = rc == SG_OK && launched != 0;
  F->t_launch += now_s() - t;
  return rc;
}

static int engine_error(sg_fits* F, int rc) {
  const char* m = sg_last_error(F->ctx);
  return fits_err(F, rc, "engine step: %s", m ? m : "error");
}

// The calling thread alternates: step the engine (launch the next step, then work on the last
// one's results, or one blocking step), then resume the fits whose columns are done -- on the
// workers when there are any, waiting for them.
static int run_sync(sg_fits* F, int64_t max_steps, size_t before) {
  for (int64_t s = 0; s < max_steps; ++s) {
    admit(F);
    if (F->pool) {
      F->pool->wait_idle();
      take_back(F);
      retire_finished(F);
    }
    if (F->active.empty() && F->pending.empty()) break;
    double t = now_s();
    int64_t fin = 0, fin2 = 0, st0[4] = {0, 0, 0, 0}, st1[4] = {0, 0, 0, 0};
    int rc = sg_engine_stats(F->ctx, st0);
    if (rc == SG_OK && F->pipelined) {
      rc = F->launched ? sg_engine_finish(F->ctx, &fin) : SG_OK;
      int launched = 0;
      const double tl = now_s();
      if (rc == SG_OK) rc = sg_engine_launch(F->ctx, &fin2, &launched);
      F->t_launch += now_s() - tl;
      F->launched = launched != 0;
    } else if (rc == SG_OK) {
      rc = sg_engine_run(F->ctx, 1, &fin);
    }
    if (rc == SG_OK) rc = sg_engine_stats(F->ctx, st1);
    if (rc == SG_OK) rc = poll_done(F);
    if (rc != SG_OK) return engine_error(F, rc);
    fin += fin2;
    const bool stepped = F->pipelined ? F->launched : st1[0] > st0[0];
    F->t_engine += now_s() - t;
    F->steps += 1;
    // Resume the fits whose awaited columns are done, oldest first.  Alone, while a step runs,
    // work for about as long as the previous step took on the GPU and leave the rest for the next
    // one: fits that started together reach their stage changes together, and doing all of that
    // host work at once would leave the GPU idle.
    double budget = -1.0;
    if (F->pipelined && F->launched && !F->pool) {
      double tm[6] = {0, 0, 0, 0, 0, 0};
      if (sg_engine_timing(F->ctx, tm) == SG_OK) {
        // 70%: a fit already started finishes past the deadline, and the next finish should not
        // find the GPU idle
        if (tm[0] >= F->gpu_ms_seen && F->gpu_ms_seen > 0) budget = 0.7 * (tm[0] - F->gpu_ms_seen) * 1e-3;
        F->gpu_ms_seen = tm[0];
      }
    }
    t = now_s();
    std::vector<std::pair<int64_t, int64_t>> ready;  // (ready_at, fit id)
    for (auto& kv : F->active) {
      Fit& f = *kv.second;
      if (!is_ready(F, f)) continue;
      if (f.ready_at < 0) f.ready_at = F->steps;
      ready.emplace_back(f.ready_at, kv.first);
    }
    std::sort(ready.begin(), ready.end());
    bool progressed = false;
    if (F->pool) {
      std::vector<Fit*> todo;
      for (const auto& r : ready) {
        Fit* f = F->active[r.second].get();
        f->busy = true;
        todo.push_back(f);
      }
      F->pool->push(todo);
      F->pool->wait_idle();
      take_back(F);
      progressed = !todo.empty();
    } else {
      for (size_t r = 0; r < ready.size(); ++r) {
        if (budget >= 0.0 && r > 0 && now_s() - t > budget) break;  // left for the next step
        advance(F, *F->active[ready[r].second]);
        progressed = true;
      }
      F->t_host += now_s() - t;
    }
    retire_finished(F);
    if (!stepped && !progressed && fin == 0 && !F->active.empty())
      return fits_err(F, SG_ERR_STATE, "engine idle while %zu fits wait for columns", F->active.size());
    if (F->finished_order.size() > before) break;
  }
  return SG_OK;
}

// Pipelined with workers: the calling thread only steps the engine.  It waits for the step in
// flight without the driver's lock, finishes it and launches the next one at once, then hands the
// fits whose columns are done to the workers, which resume them meanwhile; what they submit joins
// the next launch.  The GPU never waits for the fits' host arithmetic, only for the engine calls
// of the few fits it was in the middle of.
static int run_async(sg_fits* F, int64_t max_steps, size_t before) {
  for (int64_t s = 0; s < max_steps; ++s) {
    take_back(F);
    int64_t retired = retire_finished(F);
    admit(F);
    if (F->active.empty() && F->pending.empty()) break;
    double t = now_s();
    if (F->launched) sg_engine_wait(F->ctx);
    const double t_waited = now_s();
    F->t_wait += t_waited - t;
    // under one hold of the lock: finish the step, mark its columns done, collect the fits they
    // make ready and (without a launch wait) launch the next step
    int rc = SG_OK;
    std::vector<Fit*> todo;
    bool launch_now = F->launch_wait_s <= 0.0;
    {
      StepLock g(F);
      const double t_locked = now_s();
      F->t_lock += t_locked - t_waited;
      int64_t fin = 0;
      if (F->launched) rc = sg_engine_finish(F->ctx, &fin);
      F->launched = false;
      const double t_finished = now_s();
      F->t_finish += t_finished - t_locked;
      if (rc == SG_OK) rc = poll_done(F);
      F->t_scan += now_s() - t_finished;
      if (rc == SG_OK) {
        take_back(F);
        for (auto& kv : F->active) {
          Fit& f = *kv.second;
          if (!f.busy && !f.failed && f.phase != P_DONE && ready_locked(F, f)) {
            f.busy = true;
            todo.push_back(&f);
          }
        }
        launch_now = launch_now || todo.empty();
        if (launch_now) rc = launch_step(F);
      }
    }
    if (rc != SG_OK) return engine_error(F, rc);
    F->pool->push(todo);
    if (!launch_now) {
      // give the workers a moment, so that what they submit rides this step instead of the next
      F->pool->wait_idle_for(F->launch_wait_s);
      StepLock g(F);
      rc = launch_step(F);
      if (rc != SG_OK) return engine_error(F, rc);
    }
    F->t_engine += now_s() - t;
    F->steps += 1;
    take_back(F);
    retired += retire_finished(F);
    if (!F->launched) {
      bool busy = false;
      for (const auto& kv : F->active) busy = busy || kv.second->busy;
      if (busy) {
        // nothing on the GPU: wait for the fits being resumed to submit
        F->pool->wait_idle();
        F->idle_passes = 0;
      } else if (retired > 0 || !todo.empty() || F->active.empty()) {
        F->idle_passes = 0;
      } else if (++F->idle_passes >= 2) {
        // twice in a row nothing ran, nothing was resumed and no worker held a fit (once could be a
        // worker that submitted, or whose columns finished, after this pass launched and scanned)
        return fits_err(F, SG_ERR_STATE, "engine idle while %zu fits wait for columns", F->active.size());
      }
    } else {
      F->idle_passes = 0;
    }
    if (F->finished_order.size() > before) break;
  }
  return SG_OK;
}

static int fits_run_impl(sg_fits* F, int64_t max_steps, int64_t* n_ready) {
  if (!F) return SG_ERR_INVALID;
  const size_t before = F->finished_order.size();
  const int rc = F->pool && F->pipelined ? run_async(F, max_steps, before) : run_sync(F, max_steps, before);
  if (rc != SG_OK) return rc;
  if (n_ready) *n_ready = (int64_t)F->finished_order.size();
  return SG_OK;
}

extern "C" int sg_fits_poll(sg_fits* F, int64_t* ids, int64_t max_ids, int64_t* n_out) {
  if (!F || !n_out || (max_ids > 0 && !ids)) return SG_ERR_INVALID;
  int64_t k = 0;
  while (k < max_ids && !F->finished_order.empty()) {
    ids[k++] = F->finished_order.front();
    F->finished_order.pop_front();
  }
  *n_out = k;
  return SG_OK;
}

extern "C" int sg_fits_counts(sg_fits* F, int64_t* active, int64_t* pending, int64_t* done) {
  if (!F) return SG_ERR_INVALID;
  if (active) *active = (int64_t)F->active.size();
  if (pending) *pending = (int64_t)F->pending.size();
  if (done) *done = (int64_t)F->done_fits.size();
  return SG_OK;
}

extern "C" int sg_fits_host_times(sg_fits* F, double* t8) {
  if (!F || !t8) return SG_ERR_INVALID;
  std::lock_guard<std::mutex> g(F->mu);
  t8[0] = F->t_engine;
  t8[1] = F->t_host + (F->pool ? F->pool->busy_seconds() : 0.0);
  t8[2] = (double)F->steps;
  t8[3] = F->t_pheno;
  t8[4] = F->t_submit;
  t8[5] = F->t_fetch;
  t8[6] = F->t_dots;
  t8[7] = F->t_launch;
  return SG_OK;
}

extern "C" int sg_fits_fit_times(sg_fits* F, int64_t fit_id, double* t3) {
  if (!F || !t3) return SG_ERR_INVALID;
  std::lock_guard<std::mutex> g(F->mu);
  auto it = F->done_fits.find(fit_id);
  if (it == F->done_fits.end()) return fits_err(F, SG_ERR_NOT_FOUND, "fit %lld is not finished", (long long)fit_id);
  const Fit& f = *it->second;
  t3[0] = f.t_submit - F->t_created;
  t3[1] = f.t_admit - F->t_created;
  t3[2] = f.t_done - F->t_created;
  return SG_OK;
}

extern "C" int sg_fits_step_times(sg_fits* F, double* t4) {
  if (!F || !t4) return SG_ERR_INVALID;
  std::lock_guard<std::mutex> g(F->mu);
  t4[0] = F->t_wait;
  t4[1] = F->t_lock;
  t4[2] = F->t_finish;
  t4[3] = F->t_scan;
  return SG_OK;
}

extern "C" int sg_fits_result(sg_fits* F, int64_t fit_id, double* theta, double* alpha, double* eta,
                              double* mu, double* Y, double* cov, int32_t* iterations, int32_t* converged,
                              int64_t* column_iterations) {
  if (!F) return SG_ERR_INVALID;
  auto it = F->done_fits.find(fit_id);
  if (it == F->done_fits.end()) return fits_err(F, SG_ERR_NOT_FOUND, "fit %lld is not finished", (long long)fit_id);
  std::unique_ptr<Fit> f = std::move(it->second);
  F->done_fits.erase(it);
  if (column_iterations) *column_iterations = f->column_iterations;
  if (f->failed) return fits_err(F, f->err.code, "%s", f->err.msg.c_str());
  if (theta) {
    theta[0] = f->tau[0];
    theta[1] = f->tau[1];
  }
  if (alpha) std::memcpy(alpha, f->rc_alpha.data(), f->p * sizeof(double));
  for (int64_t s = 0; s < f->ns; ++s) {
    const int64_t i = f->idx[s];
    if (eta) eta[s] = f->rc_eta[i];
    if (mu) mu[s] = f->mu[i];
    if (Y) Y[s] = f->YX[i];
  }
  if (cov) std::memcpy(cov, f->rc_cov.data(), (size_t)f->p * f->p * sizeof(double));
  if (iterations) *iterations = f->it_used;
  if (converged) *converged = f->converged ? 1 : 0;
  return SG_OK;
}

extern "C" int sg_fits_submit(sg_fits* F, int trait, int64_t n_sub, const uint8_t* mask, const double* y,
                              const double* X, int p, const double* offset, const double* eta0,
                              const double* alpha0, double tol, int maxiter, int nrun, double tol_pcg,
                              int maxiter_pcg, double cv_cutoff, uint64_t seed, int64_t* fit_id) {
  if (!F) return SG_ERR_INVALID;
  try {
    return fits_submit_impl(F, trait, n_sub, mask, y, X, p, offset, eta0, alpha0, tol, maxiter, nrun, tol_pcg,
                            maxiter_pcg, cv_cutoff, seed, fit_id);
  } catch (const std::exception& ex) {
    return fits_err(F, SG_ERR_CUDA, "sg_fits_submit: %s", ex.what());
  }
}

extern "C" int sg_fits_run(sg_fits* F, int64_t max_steps, int64_t* n_ready) {
  if (!F) return SG_ERR_INVALID;
  try {
    return fits_run_impl(F, max_steps, n_ready);
  } catch (const std::exception& ex) {
    return fits_err(F, SG_ERR_CUDA, "sg_fits_run: %s", ex.what());
  }
}
