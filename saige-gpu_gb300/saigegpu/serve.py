"""Batched and served null-model fits on one resident GRM.

Each fit is a generator that follows the reference's algorithm step by step
(``Get_Coef`` FIT.R:2-35, ``glmmkin.ai_PCG_Rcpp_Binary`` FIT.R:79-304,
``glmmkin.ai_PCG_Rcpp_Quantitative`` FIT.R:309-549 with ``getCoefficients``
FIT.cpp:3167-3199, ``getAIScore``/``_q`` FIT.cpp:3279-3295 / 3479-3531,
``GetTrace``/``_q`` FIT.cpp:3113-3160 / 3409-3472 and the tau updates of
``fitglmmaiRPCG``/``_q`` FIT.cpp:3302-3341 / 3610-3662), all in FP64 on the
host, and *yields* its right-hand sides instead of solving them:

    ("pheno", W, tau)                       set this fit's phenotype slot
    ("submit", kind, B | None, probes, maxiter, tol) -> request ids
    ("wait", ids)                           -> the solutions (n-vectors, copied to the host)
    ("wait_ids", ids)                       -> None once finished (results stay on the GPU)
    ("probe_dots", pid, aid, seed, run0, SX) -> per-probe dot products reduced on the GPU

``Runner`` multiplexes any number of such fits onto the engine of one
``Context``: every engine step advances every in-flight column of every fit by
one PCG iteration (one pass over the GRM), columns retire on their own
stopping rule, and freed slots are refilled at the next step.  Within a fit
the batching follows the data dependencies: Y and the X columns are one block,
the 30 (+10) Hutchinson probes go with K.PY, and the P A PY solve starts as
soon as K.PY is back.  A column's arithmetic does not depend on its
neighbours, so a fit gives the same result alone or in a mix.

Sample subsets: a fit may use a mask over the cohort's samples; its vectors are
zero outside the subset and the engine solves with Sigma[S, S] built from the
cohort GRM restricted to S.  The reference instead recomputes allele
frequencies (and QC, imputation, standardisation) on each subset;
``fit_batch_exact_subsets`` does that, one GRM build per distinct subset.
"""
import concurrent.futures
import os
import threading
import time

import numpy as np

from .family import family_of
from .synth import hash3

# ------------------------------------------------------------------ generator helpers


def _solve(B, maxiter, tol):
    ids = yield ("submit", 0, B, None, maxiter, tol)
    res = yield ("wait", ids)
    return np.column_stack(res)


def _inv_sympd(A):
    A = np.triu(A) + np.triu(A, 1).T
    try:
        L = np.linalg.cholesky(A)
        Li = np.linalg.inv(L)
        return Li.T @ Li
    except np.linalg.LinAlgError:
        return np.linalg.pinv(A)


def _cal_cv(x):
    x = np.asarray(x, np.float64)
    return (x.std(ddof=1) / x.mean()) / len(x)


class FitSpec:
    """One null-model fit request.

    fit0: dict from ``prep.make_fit0`` on the subset (y, X, offset,
    linear_predictors, coefficients, family) with vectors over the subset.
    mask: bool over the cohort's n samples (None = all).
    """

    def __init__(self, fit0, trait, mask=None, tol=0.02, maxiter=20, nrun=30, tol_pcg=1e-5,
                 maxiter_pcg=500, trace_cv_cutoff=0.0025, seed=200, name=None):
        self.fit0 = fit0
        self.trait = trait
        self.mask = None if mask is None else np.asarray(mask, bool)
        self.tol, self.maxiter, self.nrun = tol, maxiter, nrun
        self.tol_pcg, self.maxiter_pcg, self.cutoff, self.seed = tol_pcg, maxiter_pcg, trace_cv_cutoff, seed
        self.name = name


class _Probes:
    """Probe vectors of the counter hash, cached per run index (identical for every fit)."""

    def __init__(self, n):
        self.n = n
        self.cache = {}

    def get(self, seed, run):
        key = (seed, run)
        if key not in self.cache:
            h = hash3(seed, run, np.arange(self.n, dtype=np.uint64))
            self.cache[key] = np.where((h >> np.uint64(63)) == 1, 1.0, -1.0)
        return self.cache[key]


def fit_generator(spec, n_cohort, probes):
    """AI-REML null fit of one phenotype as a request generator (returns the result dict)."""
    fam = family_of("binomial" if spec.trait == "binary" else "gaussian")
    quant = spec.trait != "binary"
    m = np.ones(n_cohort, bool) if spec.mask is None else spec.mask
    idx = np.nonzero(m)[0]
    n = len(idx)
    f0 = spec.fit0

    def full(v, fill=0.0):
        out = np.full(n_cohort, fill)
        out[idx] = v
        return out

    y = full(f0["y"])
    X = np.zeros((n_cohort, f0["X"].shape[1]))
    X[idx] = f0["X"]
    offset = full(np.zeros(n) if f0.get("offset") is None else f0["offset"])
    eta = full(f0["linear_predictors"])
    alpha = np.asarray(f0["coefficients"], np.float64)
    stats = {"pcg_columns": 0, "column_iterations": 0, "products": 0}

    def working(eta_):
        mu, mu_eta, var = fam.parts(eta_)
        Y = np.where(m, eta_ - offset + (y - mu) / mu_eta, 0.0)
        W = np.where(m, (mu_eta / np.sqrt(var)) ** 2, 1.0) if not quant else np.ones_like(Y)
        return mu, Y, W

    def get_coefficients(Y, W, tau):
        yield ("pheno", W, tau)
        S = yield from _solve(np.column_stack([Y, X]), spec.maxiter_pcg, spec.tol_pcg)
        SY, SX = S[:, 0], S[:, 1:]
        cov = _inv_sympd(X.T @ SX)
        al = cov @ (SX.T @ Y)
        et = np.where(m, Y - tau[0] * (SY - SX @ al) / W, 0.0)
        return dict(Sigma_iY=SY, Sigma_iX=SX, cov=cov, alpha=al, eta=et)

    def get_coef(tau, alpha0, eta0):
        mu, Y, W = working(eta0)
        for _ in range(spec.maxiter):
            rc = yield from get_coefficients(Y, W, tau)
            al = rc["alpha"]
            et = rc["eta"] + offset
            mu, Y, W = working(et)
            if np.max(np.abs(al - alpha0) / (np.abs(al) + np.abs(alpha0) + 0.1)) < 0.1:
                break
            alpha0 = al
        return dict(Y=Y, alpha=al, eta=et, W=W, cov=rc["cov"], Sigma_iY=rc["Sigma_iY"],
                    Sigma_iX=rc["Sigma_iX"], mu=mu)

    def ai_score(rc, tau):
        Y, W, SY, SX = rc["Y"], rc["W"], rc["Sigma_iY"], rc["Sigma_iX"]
        yield ("pheno", W, tau)  # getAIScore solves with Get_Coef's updated weights (FIT.R:142, :186)
        cov = _inv_sympd(X.T @ SX) if quant else rc["cov"]
        PY = SY - SX @ (cov @ (SX.T @ Y))
        # K PY rides with the first probe block
        apy_id = yield ("submit", 1, PY[:, None], None, 1, 0.0)
        pid = yield ("submit", 0, None, (spec.seed, 0, spec.nrun), spec.maxiter_pcg, spec.tol_pcg)
        # K u is fixed for the fit (same probes, same sample mask): -1 marks a cached product
        aid = yield ("probe_products", spec.seed, 0, spec.nrun)
        APY = (yield ("wait", apy_id))[0]
        rhs = np.column_stack([APY, PY]) if quant else APY[:, None]
        sid = yield ("submit", 0, rhs, None, spec.maxiter_pcg, spec.tol_pcg)
        t1, t0 = [], []
        run0, k = 0, spec.nrun
        p = SX.shape[1]
        while True:
            yield ("wait_ids", list(pid) + [a for a in aid if a >= 0])
            # t1 = Au.Pu, t0 = u.Pu with Pu = Su - SX cov SX'u, from device-side dot products
            D = yield ("probe_dots", pid, aid, spec.seed, run0, SX)
            b, c = D[:, 2:2 + p], D[:, 2 + p:2 + 2 * p]
            t1.extend(D[:, 0] - np.einsum("ij,jk,ik->i", b, cov, c))
            t0.extend(D[:, 1] - np.einsum("ij,jk,ik->i", c, cov, c))
            if _cal_cv(t1) > spec.cutoff or (quant and _cal_cv(t0) > spec.cutoff):
                run0, k = run0 + k, 10
                pid = yield ("submit", 0, None, (spec.seed, run0, k), spec.maxiter_pcg, spec.tol_pcg)
                aid = yield ("probe_products", spec.seed, run0, k)
                continue
            break
        S = np.column_stack((yield ("wait", sid)))
        PAPY = S[:, 0] - SX @ (cov @ (SX.T @ S[:, 0]))
        out = dict(YPAPY=float(PY @ APY), Trace=float(np.mean(t1)), PY=PY, nprobe=len(t1))
        if quant:
            PA0PY = S[:, 1] - SX @ (cov @ (SX.T @ S[:, 1]))
            out["YPA0PY"] = float(PY @ PY)
            out["Trace"] = np.array([np.mean(t0), np.mean(t1)])
            out["AI"] = np.array([[PY @ PA0PY, PY @ PAPY], [PY @ PAPY, APY @ PAPY]])
        else:
            out["AI"] = float(APY @ PAPY)
        return out

    def tau_step(rc, tau):
        re = yield from ai_score(rc, tau)
        tau0 = np.array(tau, np.float64)
        if not quant:  # fitglmmaiRPCG (FIT.cpp:3302-3341)
            dtau = (re["YPAPY"] - re["Trace"]) / re["AI"]
            t = tau0.copy()
            t[1] = tau0[1] + dtau
            t[t < spec.tol] = 0.0
            step = 1.0
            while t[1] < 0.0:
                step *= 0.5
                t[1] = tau0[1] + step * dtau
            t[t < spec.tol] = 0.0
            return t
        zero = tau0 < spec.tol  # fitglmmaiRPCG_q (FIT.cpp:3610-3662)
        score = np.array([re["YPA0PY"] - re["Trace"][0], re["YPAPY"] - re["Trace"][1]])
        dtau = np.linalg.solve(re["AI"], score)
        t = tau0 + dtau
        t[zero & (t < spec.tol)] = 0.0
        step = 1.0
        while t[0] < 0.0 or t[1] < 0.0:
            step *= 0.5
            t = tau0 + step * dtau
            t[zero & (t < spec.tol)] = 0.0
        t[t < spec.tol] = 0.0
        return t

    # ---------------- glmmkin.ai_PCG_Rcpp_* main loop
    alpha0 = alpha
    eta0 = eta
    if quant:
        _, Y0, _ = working(eta)
        tau = np.array([1.0, 0.0])
        if abs(np.var(Y0[idx], ddof=1)) < 0.1:
            raise ValueError("variance of the phenotype is much smaller than 1")
    else:
        tau = np.array([1.0, 0.1])
    tau0 = tau.copy()
    rc = yield from get_coef(tau, alpha0, eta0)
    re = yield from ai_score(rc, tau)
    if quant:
        tau[1] = max(0.0, tau0[1] + tau0[1] ** 2 * (re["YPAPY"] - re["Trace"][1]) / n)
        tau[0] = max(0.0, tau0[0] + tau0[0] ** 2 * (re["YPA0PY"] - re["Trace"][0]) / n)
    else:
        tau[1] = max(0.0, tau0[1] + tau0[1] ** 2 * (re["YPAPY"] - re["Trace"]) / n)
    it_used = 0
    for i in range(1, spec.maxiter + 1):
        it_used = i
        alpha0 = rc["alpha"] if not quant else alpha
        tau0 = tau.copy()
        eta0 = eta
        rc = yield from get_coef(tau, alpha0, eta0)
        tau = yield from tau_step(rc, tau)
        alpha, eta = rc["alpha"], rc["eta"]
        if quant and tau[0] <= 0:
            raise ValueError("the first variance component parameter estimate is 0")
        if tau[1] <= 0 if quant else tau[1] == 0:
            break
        if np.max(np.abs(tau - tau0) / (np.abs(tau) + np.abs(tau0) + spec.tol)) < spec.tol:
            break
        if np.max(tau) > spec.tol ** (-2):
            it_used = spec.maxiter
            break
    rc = yield from get_coef(tau, alpha, eta)
    return dict(theta=tau, coefficients=rc["alpha"], linear_predictors=rc["eta"][idx],
                fitted_values=rc["mu"][idx], Y=rc["Y"][idx], residuals=(y - rc["mu"])[idx],
                cov=rc["cov"], converged=it_used < spec.maxiter, iterations=it_used, n=n)


def loco_generator(spec, fit, n_cohort):
    """Get_Coef_LOCO (FIT.R:40-73) for one phenotype while the engine leaves a chromosome out,
    started from the full fit's tau, alpha and eta (FIT.R:254-297)."""
    fam = family_of("binomial" if spec.trait == "binary" else "gaussian")
    quant = spec.trait != "binary"
    m = np.ones(n_cohort, bool) if spec.mask is None else spec.mask
    idx = np.nonzero(m)[0]
    f0 = spec.fit0

    def full(v):
        out = np.zeros(n_cohort)
        out[idx] = v
        return out

    y = full(f0["y"])
    X = np.zeros((n_cohort, f0["X"].shape[1]))
    X[idx] = f0["X"]
    offset = full(np.zeros(len(idx)) if f0.get("offset") is None else f0["offset"])
    tau = np.asarray(fit["theta"], np.float64)
    alpha0 = np.asarray(fit["coefficients"], np.float64)
    eta0 = full(fit["linear_predictors"])

    def working(eta_):
        mu, mu_eta, var = fam.parts(eta_)
        Y = np.where(m, eta_ - offset + (y - mu) / mu_eta, 0.0)
        W = np.where(m, (mu_eta / np.sqrt(var)) ** 2, 1.0) if not quant else np.ones_like(Y)
        return mu, Y, W

    mu, Y, W = working(eta0)
    for _ in range(spec.maxiter):
        yield ("pheno", W, tau)
        S = yield from _solve(np.column_stack([Y, X]), spec.maxiter_pcg, spec.tol_pcg)
        SY, SX = S[:, 0], S[:, 1:]
        cov = _inv_sympd(X.T @ SX)
        al = cov @ (SX.T @ Y)
        et = np.where(m, Y - tau[0] * (SY - SX @ al) / W, 0.0) + offset
        mu, Y, W = working(et)
        if np.max(np.abs(al - alpha0) / (np.abs(al) + np.abs(alpha0) + 0.1)) < 0.1:
            break
        alpha0 = al
    return dict(isLOCO=True, coefficients=al, linear_predictors=et[idx], fitted_values=mu[idx],
                Y=Y[idx], residuals=(y - mu)[idx], cov=cov)


def loco_ranges(chrom_of_grm_markers):
    """Per-autosome [begin, end] of the GRM markers (updateChrStartEndIndexVec, Util.R:29-65);
    None for chromosomes without markers.  Markers must be ordered by chromosome.  Given every .bim
    marker's chromosome, the same ranges index the .bim markers (``fit_loco(..., bim=True)``)."""
    chrom = np.asarray(chrom_of_grm_markers)
    out = {}
    last_end = -1
    for c in range(1, 23):
        w = np.nonzero(chrom == c)[0]
        if len(w) == 0:
            out[c] = None
            continue
        b, e = int(w.min()), int(w.max())
        if b <= last_end:
            raise ValueError("chromosomes need to be ordered from 1 to 22 in the bim file")
        last_end = e
        out[c] = (b, e)
    return out


def fit_loco(ctx, specs, fits, ranges, max_columns=1024, bim=False):
    """LOCO results per chromosome for fitted phenotypes: {chrom: [result or None per spec]}.

    ``ranges`` ({chrom: (begin, end) or None}, from ``loco_ranges``) index the GRM markers, or with
    ``bim`` the .bim markers; the subset-exact engines take .bim ranges only, since each phenotype's
    GRM markers are those passing QC over its own samples (the chromosome's markers among them leave
    its GRM)."""
    out = {}
    set_range = ctx.loco_set_bim if bim else ctx.loco_set
    for c, rng in ranges.items():
        if rng is None:
            out[c] = [dict(isLOCO=False) for _ in specs]
            continue
        set_range(rng[0], rng[1])
        try:
            r = Runner(ctx, max_columns, max(1, len(specs)))
            ids = []
            for spec, fit in zip(specs, fits):
                jid = r._next
                r._next += 1
                slot = r.free_slots.pop()
                job = _Job(jid, spec, loco_generator(spec, fit, r.n), slot, time.perf_counter())
                r.jobs[jid] = job
                r._advance(job, None)
                ids.append(jid)
            try:
                r.run()
            finally:
                r.close()
            by = {j.jid: j for j in r.finished}
            out[c] = [by[i].result if by[i].error is None else by[i].error for i in ids]
        finally:
            ctx.loco_clear()
    return out


# ------------------------------------------------------------------ runner


class _Job:
    def __init__(self, jid, spec, gen, slot, t_arrive):
        self.jid, self.spec, self.gen, self.slot = jid, spec, gen, slot
        self.waiting = None
        self.results = {}
        self.t_arrive = t_arrive
        self.t_start = None
        self.t_done = None
        self.result = None
        self.error = None
        self.column_iterations = 0
        self.columns = 0
        self.ready_at = None  # step at which every awaited column was done


class Runner:
    """Continuous batching of many null-model fits over one engine."""

    def __init__(self, ctx, max_columns=2048, max_phenos=64, min_columns_per_fit=2 * (30 + 10) + 8,
                 pipelined=True, workers=None):
        if max_columns < min_columns_per_fit:
            # a fit's trace stage keeps ~2 (nrun + 10) + 4 columns in flight at once
            raise ValueError("max_columns=%d is below one fit's working set (%d)" % (max_columns, min_columns_per_fit))
        self.ctx = ctx
        self.n = ctx.n
        ctx.engine_reserve(max_columns, max_phenos)
        if hasattr(ctx, "engine_hold_results"):
            ctx.engine_hold_results(True)  # probe results are reduced on the device, not copied
        self.max_columns = max_columns
        self.free_slots = list(range(max_phenos))[::-1]
        self.jobs = {}
        self.owner = {}          # request id -> job id
        self.done = set()        # finished request ids (results resident on the GPU)
        self.probes = _Probes(self.n)
        self.finished = []
        self._next = 0
        self.inflight_columns = 0
        # pipelined: step k+1 runs on the GPU while the fits consume step k's results (their new
        # columns join step k+2)
        self.pipelined = bool(pipelined) and hasattr(ctx, "engine_launch")
        self._launched = False
        self._steps = 0
        self._gpu_ms = 0.0
        self._lock = threading.RLock()
        # host threads that run the fits' driver math while the main thread steps the engine; one by
        # default: measured on the 16-core Arm host, 8 threads made the numpy driver 7x slower in
        # total (GIL contention) and end-to-end throughput fell from 89.6k to 70.0k fits/hr
        self.workers = max(1, int(workers if workers is not None else 1))
        self._pool = None
        if self.workers > 1:
            init = getattr(ctx, "make_current", None)
            self._pool = concurrent.futures.ThreadPoolExecutor(self.workers, initializer=init)
        # wall-clock seconds by activity (engine steps incl. their sync, result copies, driver math)
        self.t = {"engine": 0.0, "fetch": 0.0, "probe_dots": 0.0, "pheno": 0.0, "submit": 0.0, "driver": 0.0}

    # -- admission
    def can_admit(self, spec):
        """Admit a fit only if its peak working set fits beside the columns already in flight
        (results stay on the device until consumed, so oversubscribing could stall)."""
        need = 2 * (spec.nrun + 10) + 8
        return bool(self.free_slots) and self.inflight_columns + need <= self.max_columns

    def submit(self, spec, t_arrive=None):
        if not self.free_slots:
            raise RuntimeError("no free phenotype slot")
        jid = self._next
        self._next += 1
        slot = self.free_slots.pop()
        if hasattr(self.ctx, "engine_probe_cache_clear"):
            self.ctx.engine_probe_cache_clear(slot)  # a new sample mask takes this slot
        job = _Job(jid, spec, fit_generator(spec, self.n, self.probes), slot,
                   time.perf_counter() if t_arrive is None else t_arrive)
        job.t_start = time.perf_counter()
        self.jobs[jid] = job
        self._advance(job, None)
        return jid

    # -- generator plumbing
    def _advance(self, job, value):
        """Run a fit's generator until it waits for columns or ends.  The generator's own numpy
        work runs outside the lock (worker threads overlap it); every engine call and every
        change to the runner's bookkeeping happens under it."""
        gen = job.gen
        clock = time.perf_counter
        try:
            while True:
                t0 = clock()
                op = gen.send(value)
                with self._lock:
                    self.t["driver"] += clock() - t0
                    value, waiting = self._do_op(job, op)
                    if waiting:
                        return
        except StopIteration as st:
            with self._lock:
                job.result = st.value
                self._finish(job)
        except Exception as ex:  # the fit failed: release its slot, keep the others running
            with self._lock:
                job.error = ex
                self._finish(job)

    def _do_op(self, job, op):
        """One engine request of a generator (lock held); returns (value to send, waiting)."""
        clock = time.perf_counter
        t1 = clock()
        kind = op[0]
        if kind == "pheno":
            _, W, tau = op
            self.ctx.engine_set_pheno(job.slot, W, tau, job.spec.mask)
            self.t["pheno"] += clock() - t1
            return None, False
        if kind == "submit":
            _, k, B, probe, maxiter, tol = op
            if probe is None:
                ids = self.ctx.engine_submit(job.slot, k, B, maxiter, tol)
            else:
                seed, run0, cnt = probe
                ids = self.ctx.engine_submit_probes(job.slot, k, seed, run0, cnt, maxiter, tol)
            self.t["submit"] += clock() - t1
            for i in ids:
                self.owner[int(i)] = job.jid
            job.columns += len(ids)
            self.inflight_columns += len(ids)
            return [int(i) for i in ids], False
        if kind in ("wait", "wait_ids"):
            ids = op[1]
            if all(i in self.done for i in ids):
                return self._resolve(job, kind, ids), False
            job.waiting = (kind, ids)
            return None, True
        if kind == "probe_products":
            _, seed, run0, cnt = op
            value = [-1] * cnt
            j = 0
            while j < cnt:  # submit maximal runs of uncached probes as blocks
                if self.ctx.engine_probe_cached(job.slot, seed, run0 + j):
                    j += 1
                    continue
                j1 = j
                while j1 < cnt and not self.ctx.engine_probe_cached(job.slot, seed, run0 + j1):
                    j1 += 1
                ids = self.ctx.engine_submit_probes(job.slot, 1, seed, run0 + j, j1 - j, 1, 0.0)
                for q, i in enumerate(ids):
                    value[j + q] = int(i)
                    self.owner[int(i)] = job.jid
                job.columns += len(ids)
                self.inflight_columns += len(ids)
                j = j1
            self.t["submit"] += clock() - t1
            return value, False
        if kind == "probe_dots":
            _, pid, aid, seed, run0, SX = op
            D, its = self.ctx.engine_probe_dots(job.slot, pid, aid, seed, run0, SX)
            self.t["probe_dots"] += clock() - t1
            job.column_iterations += int(np.sum(its)) + sum(1 for a in aid if a >= 0)
            for i in list(pid) + [a for a in aid if a >= 0]:
                self.done.discard(i)
                self.owner.pop(i, None)
            return D, False
        raise RuntimeError("unknown op %r" % (kind,))

    def _resume(self, job, kind, wids):
        with self._lock:
            value = self._resolve(job, kind, wids)
        self._advance(job, value)

    def _resolve(self, job, kind, ids):
        if kind == "wait_ids":
            return None
        t0 = time.perf_counter()
        out = []
        for rid in ids:
            x, it = self.ctx.engine_fetch(rid)
            self.done.discard(rid)
            self.owner.pop(rid, None)
            job.column_iterations += it
            out.append(x)
        self.t["fetch"] += time.perf_counter() - t0
        return out

    def _finish(self, job):
        job.t_done = time.perf_counter()
        for rid, jid in list(self.owner.items()):
            if jid == job.jid:
                try:
                    self.ctx.engine_cancel(rid)
                except Exception:
                    pass
                self.owner.pop(rid, None)
                self.done.discard(rid)
        self.free_slots.append(job.slot)
        del self.jobs[job.jid]
        self.finished.append(job)

    def step(self):
        """One engine step; resume every fit whose awaited columns are complete."""
        t0 = time.perf_counter()
        if self.pipelined:
            if self._launched:
                self.ctx.engine_finish()
            try:
                self._launched, _ = self.ctx.engine_launch()
            except Exception:
                # queued columns found every column holding a result: resume every ready fit (they
                # consume their results) and try once more
                if not self._resume_all_ready():
                    raise
                self._launched, _ = self.ctx.engine_launch()
        else:
            self.ctx.engine_run(1)
        ids = self.ctx.engine_poll()
        t1 = time.perf_counter()
        self.t["engine"] += t1 - t0
        if self.pipelined and not self._launched and len(ids) == 0:
            stuck = [j.jid for j in self.jobs.values()
                     if j.waiting is not None and not all(i in self.done for i in j.waiting[1])]
            if stuck:
                raise RuntimeError("engine idle while fits %s wait for columns" % stuck)
        for rid in ids:
            rid = int(rid)
            if rid not in self.owner:
                continue
            self.done.add(rid)
            self.inflight_columns -= 1
        self._steps += 1
        ready = []
        for j in self.jobs.values():
            if j.waiting is not None and all(i in self.done for i in j.waiting[1]):
                if j.ready_at is None:
                    j.ready_at = self._steps
                ready.append(j)
        ready.sort(key=lambda j: (j.ready_at, j.jid))
        # While a step runs, resume fits for about as long as the previous step took on the GPU and
        # leave the rest for the next one: fits that started together reach their stage changes
        # together, and doing all that host work at once would leave the GPU idle.
        budget = self._host_budget() if (self.pipelined and self._launched) else None
        if self._pool is None:
            for k, job in enumerate(ready):
                if budget is not None and k > 0 and time.perf_counter() - t1 > budget:
                    break
                (kind, wids), job.waiting = job.waiting, None
                job.ready_at = None
                self._resume(job, kind, wids)
            return len(ids)
        # up to `workers` fits at a time; stop starting new ones once the budget is spent
        pending, running, started = list(ready), set(), 0
        while pending or running:
            while pending and len(running) < self.workers and (
                    budget is None or started == 0 or time.perf_counter() - t1 <= budget):
                job = pending.pop(0)
                (kind, wids), job.waiting = job.waiting, None
                job.ready_at = None
                running.add(self._pool.submit(self._resume, job, kind, wids))
                started += 1
            if not running:
                break
            finished, running = concurrent.futures.wait(running, return_when=concurrent.futures.FIRST_COMPLETED)
            for f in finished:
                f.result()
        return len(ids)

    def close(self):
        if self._pool is not None:
            self._pool.shutdown(wait=True)
            self._pool = None

    def _resume_all_ready(self):
        ready = [j for j in self.jobs.values()
                 if j.waiting is not None and all(i in self.done for i in j.waiting[1])]
        for job in ready:
            (kind, wids), job.waiting = job.waiting, None
            job.ready_at = None
            self._resume(job, kind, wids)
        return bool(ready)

    def _host_budget(self):
        """GPU seconds of the last finished step (None when the engine does not time its steps)."""
        timing = getattr(self.ctx, "engine_timing", None)
        if timing is None:
            return None
        total = timing()["step_ms"]
        last = total - self._gpu_ms
        self._gpu_ms = total
        return max(last, 0.0) * 1e-3 if last > 0 else None

    def run(self, max_steps=1 << 30):
        steps = 0
        while self.jobs and steps < max_steps:
            self.step()
            steps += 1
        self.drain()
        return steps

    def drain(self):
        """Wait for a launched step whose columns no fit awaits any more (cancelled or failed fits)."""
        if self._launched:
            self.ctx.engine_finish()
            self._launched = False
            for rid in self.ctx.engine_poll():
                if int(rid) in self.owner:
                    self.done.add(int(rid))
                    self.inflight_columns -= 1

    def cancel(self, jid):
        job = self.jobs.get(jid)
        if job is not None:
            job.error = RuntimeError("cancelled")
            job.gen.close()
            self._finish(job)


def columns_for(specs):
    """Engine columns that hold every fit's peak working set at once (trace stage: probes,
    their products, K.PY and the P A PY solves)."""
    need = sum(2 * (s.nrun + 10) + 8 for s in specs)
    return int(-(-need // 256) * 256)


def fit_batch(ctx, specs, max_columns=None, max_phenos=None, pipelined=True, workers=None):
    """Fit all ``specs`` together; returns their result dicts (or exceptions) in order.  With
    max_phenos below len(specs), at most that many run at once."""
    conc = max_phenos or max(1, len(specs))
    max_columns = max(max_columns or 0, columns_for(sorted(specs, key=lambda sp: -sp.nrun)[:conc]))
    r = Runner(ctx, max_columns, conc, pipelined=pipelined, workers=workers)
    try:
        ids = [r.submit(s) for s in specs]
        r.run()
    finally:
        r.close()
    by = {j.jid: j for j in r.finished}
    jobs = [by[i] for i in ids]
    for j in jobs:
        j.host_times = r.t
    return [by[i].result if by[i].error is None else by[i].error for i in ids], jobs


def fit_batch_exact_subsets(ctx, specs, max_columns=None, max_phenos=None, pipelined=True):
    """Fits whose sample masks differ run on GRMs rebuilt for their own subsets.

    Specs are grouped by mask; each group's samples become the cohort (``Context.subset_cohort``:
    allele frequencies, QC, imputation, standardisation and K recomputed over the subset, as the
    reference's setgeno does for a phenotype observed on those samples) and the group is fitted as
    full-cohort fits; the original cohort and its GRM are restored at the end.  One GRM build per
    distinct subset.  Returns (results, jobs) in the order of ``specs``."""
    import copy
    groups = {}
    for i, sp in enumerate(specs):
        key = None if sp.mask is None or bool(np.all(sp.mask)) else np.packbits(sp.mask).tobytes()
        groups.setdefault(key, []).append(i)
    results, jobs = [None] * len(specs), [None] * len(specs)
    order = sorted(groups, key=lambda k: k is not None)  # the resident full cohort first
    prev = None
    try:
        for key in order:
            idx = groups[key]
            if key is not None:
                if prev is None:
                    prev = ctx.cohort()
                keep = np.asarray(specs[idx[0]].mask, bool)
                sub = prev["sub"][keep]
                fam_mask = np.zeros_like(prev["mask"])
                fam_mask[sub - 1] = prev["mask"][sub - 1]
                ctx.set_cohort(sub, fam_mask, prev["grm"], prev["mode"])
            sub_specs = []
            for i in idx:
                sp = copy.copy(specs[i])
                sp.mask = None
                sub_specs.append(sp)
            res, jb = fit_batch(ctx, sub_specs, max_columns, max_phenos, pipelined)
            for i, r, j in zip(idx, res, jb):
                results[i], jobs[i] = r, j
    finally:
        if prev is not None:
            ctx.set_cohort(prev["sub"], prev["mask"], prev["grm"], prev["mode"])
    return results, jobs


def serve(ctx, arrivals, max_columns=2048, max_phenos=64, clock=time.perf_counter, pipelined=True,
          workers=None):
    """Serve a stream of (t_arrival_seconds, FitSpec): admit as slots and columns free up.

    Returns the finished jobs (with t_arrive / t_start / t_done) in completion order.
    """
    r = Runner(ctx, max_columns, max_phenos, pipelined=pipelined, workers=workers)
    pending = sorted(arrivals, key=lambda a: a[0])
    t0 = clock()
    k = 0
    while k < len(pending) or r.jobs:
        now = clock() - t0
        while k < len(pending) and pending[k][0] <= now and r.can_admit(pending[k][1]):
            r.submit(pending[k][1], t_arrive=t0 + pending[k][0])
            k += 1
        if r.jobs:
            r.step()
        elif k < len(pending):
            r.drain()
            time.sleep(max(0.0, min(0.01, pending[k][0] - now)))
    r.drain()
    r.close()
    return r.finished
