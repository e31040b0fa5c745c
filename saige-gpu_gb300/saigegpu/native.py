"""Batched null-model fits driven from native code (``sg_fits_*`` in ``csrc/fits.cu``).

Same algorithm and result dictionaries as ``serve.fit_generator`` run by ``serve.Runner`` --
glmmkin.ai_PCG_Rcpp_Binary / _Quantitative (src/SAIGE/R/SAIGE_fitGLMM_fast.R:79-549) over the
continuous-batching engine -- but the per-fit driver (working vectors, coefficients, traces, tau
updates) runs in C++ next to the engine, so the host keeps up with the GPU.
"""
import ctypes as C
import time

import numpy as np

from . import _lib as L


def _p(a, t):
    return a.ctypes.data_as(t) if a is not None else None


class NativeFits:
    """One ``sg_fits`` driver over a context's engine."""

    def __init__(self, ctx, max_columns, max_fits, pipelined=True, threads=None, lib=None, launch_wait_ms=None):
        """threads: host threads for the fits' arithmetic (None: half the cores, at most 8).
        lib: a library exporting the sg_fits_* ABI other than libsaigegpu (bound with
        ``_lib.bind``); ctx then only needs ``_h`` and ``last_error()``.
        launch_wait_ms: see ``sg_fits_set_launch_wait`` (None: the library default)."""
        self.ctx = ctx
        self._L = L.load() if lib is None else lib
        h = C.c_void_p()
        rc = self._L.sg_fits_create(ctx._h, int(max_columns), int(max_fits), int(bool(pipelined)), C.byref(h))
        if rc != 0:
            raise L.SaigeGpuError(rc, ctx.last_error())
        self._h = h
        self.specs = {}
        if threads is not None:
            self._check(self._L.sg_fits_set_threads(self._h, int(threads)))
        if launch_wait_ms is not None:
            self._check(self._L.sg_fits_set_launch_wait(self._h, float(launch_wait_ms)))

    def close(self):
        if getattr(self, "_h", None):
            self._L.sg_fits_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            raise L.SaigeGpuError(rc, (self._L.sg_fits_last_error(self._h) or b"").decode())

    def submit(self, spec):
        """Queue one ``serve.FitSpec``; returns its fit id."""
        f0 = spec.fit0
        y = np.ascontiguousarray(f0["y"], np.float64)
        X = np.asfortranarray(np.asarray(f0["X"], np.float64))
        ns, p = X.shape
        off = None if f0.get("offset") is None else np.ascontiguousarray(f0["offset"], np.float64)
        eta = np.ascontiguousarray(f0["linear_predictors"], np.float64)
        alpha = np.ascontiguousarray(f0["coefficients"], np.float64)
        mask = None if spec.mask is None else np.ascontiguousarray(spec.mask, np.uint8)
        fid = C.c_int64()
        self._check(self._L.sg_fits_submit(
            self._h, 0 if spec.trait == "binary" else 1, int(ns), _p(mask, L.P_u8), _p(y, L.P_f64),
            X.ctypes.data_as(L.P_f64), int(p), _p(off, L.P_f64), _p(eta, L.P_f64), _p(alpha, L.P_f64),
            float(spec.tol), int(spec.maxiter), int(spec.nrun), float(spec.tol_pcg), int(spec.maxiter_pcg),
            float(spec.cutoff), int(spec.seed), C.byref(fid)))
        self.specs[fid.value] = (spec, ns, p)
        return fid.value

    def run(self, max_steps=1 << 30):
        n = C.c_int64()
        self._check(self._L.sg_fits_run(self._h, int(max_steps), C.byref(n)))
        return n.value

    def poll(self, max_ids=4096):
        ids = np.empty(max_ids, np.int64)
        n = C.c_int64()
        self._check(self._L.sg_fits_poll(self._h, ids.ctypes.data_as(L.P_i64), int(max_ids), C.byref(n)))
        return [int(i) for i in ids[:n.value]]

    def counts(self):
        a, p, d = C.c_int64(), C.c_int64(), C.c_int64()
        self._check(self._L.sg_fits_counts(self._h, C.byref(a), C.byref(p), C.byref(d)))
        return a.value, p.value, d.value

    def host_times(self):
        """Seconds: engine stepping, driver work (and its pheno / submit / fetch / probe_dots parts)."""
        t = np.zeros(8)
        self._check(self._L.sg_fits_host_times(self._h, t.ctypes.data_as(L.P_f64)))
        u = np.zeros(4)
        self._check(self._L.sg_fits_step_times(self._h, u.ctypes.data_as(L.P_f64)))
        return {"engine": t[0], "driver": t[1], "steps": int(t[2]), "pheno": t[3], "submit": t[4],
                "fetch": t[5], "probe_dots": t[6], "launch": t[7], "step_wait": u[0], "lock_wait": u[1],
                "finish": u[2], "mark_done": u[3]}

    def fit_times(self, fid):
        """(added, admitted, finished) seconds since the driver was created, for a finished fit not
        yet collected by ``result``."""
        t = np.zeros(3)
        self._check(self._L.sg_fits_fit_times(self._h, int(fid), t.ctypes.data_as(L.P_f64)))
        return float(t[0]), float(t[1]), float(t[2])

    def result(self, fid):
        """(result dict, column iterations); the dict has the keys of ``serve.fit_generator``'s."""
        spec, ns, p = self.specs.pop(fid)
        theta, alpha = np.zeros(2), np.zeros(p)
        eta, mu, Y = np.zeros(ns), np.zeros(ns), np.zeros(ns)
        cov = np.zeros((p, p), order="F")
        it, conv, colit = C.c_int32(), C.c_int32(), C.c_int64()
        rc = self._L.sg_fits_result(self._h, int(fid), _p(theta, L.P_f64), _p(alpha, L.P_f64), _p(eta, L.P_f64),
                                    _p(mu, L.P_f64), _p(Y, L.P_f64), cov.ctypes.data_as(L.P_f64),
                                    C.byref(it), C.byref(conv), C.byref(colit))
        if rc != 0:
            return L.SaigeGpuError(rc, (self._L.sg_fits_last_error(self._h) or b"").decode()), colit.value
        y = np.asarray(spec.fit0["y"], np.float64)
        return dict(theta=theta, coefficients=alpha, linear_predictors=eta, fitted_values=mu, Y=Y,
                    residuals=y - mu, cov=np.ascontiguousarray(cov), converged=bool(conv.value),
                    iterations=int(it.value), n=ns), colit.value


class _Job:
    def __init__(self, jid, spec, t_arrive):
        self.jid, self.spec = jid, spec
        self.t_arrive, self.t_start, self.t_done = t_arrive, time.perf_counter(), None
        self.result = self.error = None
        self.column_iterations = 0
        self.columns = 0
        self.host_times = {}
        self.service_s = None  # admission to a slot -> finished (native driver)


def fit_batch(ctx, specs, max_columns=None, max_phenos=None, pipelined=True, threads=None, lib=None,
              launch_wait_ms=None):
    """Fit all ``specs`` together in native code; returns (results or exceptions, jobs) in order.
    With max_phenos below len(specs) at most that many fits run at once, the others entering as
    running ones finish (a stream through max_phenos phenotype slots)."""
    from .serve import columns_for
    conc = max_phenos or max(1, len(specs))
    # engine columns for the conc largest working sets that can run together
    widest = sorted(specs, key=lambda sp: -sp.nrun)[:conc]
    max_columns = max(max_columns or 0, columns_for(widest))
    drv = NativeFits(ctx, max_columns, conc, pipelined, threads, lib, launch_wait_ms)
    try:
        jobs = {}
        for s in specs:
            fid = drv.submit(s)
            jobs[fid] = _Job(fid, s, time.perf_counter())
        order = list(jobs)
        left = len(jobs)
        while left:
            drv.run()
            for fid in drv.poll():
                j = jobs[fid]
                j.t_done = time.perf_counter()
                # service time: from the fit's admission to a phenotype slot to its end
                t_add, t_adm, t_fin = drv.fit_times(fid)
                j.service_s = t_fin - t_adm
                res, j.column_iterations = drv.result(fid)
                if isinstance(res, Exception):
                    j.error = res
                else:
                    j.result = res
                left -= 1
        times = drv.host_times()
    finally:
        drv.close()
    out = []
    for fid in order:
        jobs[fid].host_times = times
        out.append(jobs[fid].result if jobs[fid].error is None else jobs[fid].error)
    return out, [jobs[f] for f in order]


def serve(ctx, arrivals, max_columns=2048, max_phenos=64, clock=time.perf_counter, pipelined=True,
          threads=None, lib=None, launch_wait_ms=None):
    """Serve (t_arrival_seconds, FitSpec) requests with the native driver; returns the finished jobs
    (t_arrive / t_start / t_done) in completion order."""
    drv = NativeFits(ctx, max_columns, max_phenos, pipelined, threads, lib, launch_wait_ms)
    pending = sorted(arrivals, key=lambda a: a[0])
    jobs, finished = {}, []
    t0 = clock()
    k = 0
    try:
        while k < len(pending) or jobs:
            now = clock() - t0
            while k < len(pending) and pending[k][0] <= now:
                fid = drv.submit(pending[k][1])
                jobs[fid] = _Job(fid, pending[k][1], t0 + pending[k][0])
                k += 1
            if jobs:
                drv.run(1)
                for fid in drv.poll():
                    j = jobs.pop(fid)
                    j.t_done = clock()
                    res, j.column_iterations = drv.result(fid)
                    if isinstance(res, Exception):
                        j.error = res
                    else:
                        j.result = res
                    finished.append(j)
            elif k < len(pending):
                time.sleep(max(0.0, min(0.01, pending[k][0] - now)))
    finally:
        drv.close()
    return finished
