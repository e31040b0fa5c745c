"""The native fit driver (csrc/fits.cu) on the CPU, over a CPU stand-in of the engine.

fits.cu is plain host C++ and a client of the engine's C ABI only, so it links against
tests/fake_engine/fake_engine.cpp (dense FP64 K, the engine's request / slot / probe-cache
semantics, emulated step time) into a test library.  This covers the driver's state machines
(Get_Coef, getAIScore, GetTrace with the CV-driven extra probes, tau updates), admission of queued
fits into free slots, and its threading: worker threads resuming fits while the calling thread
steps (pipelined), the calling thread alone, and blocking steps must give identical fits, equal to
the oracle's.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from oracle import aireml, plink
from saigegpu import _lib as L
from saigegpu import native, prep, serve, synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def fake_lib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("fake") / "libfitsfake.so")
    cmd = ["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-pthread", "-Wl,--no-undefined",
           "-x", "c++", os.path.join(ROOT, "saige-gpu_gb300", "csrc", "fits.cu"),
           "-x", "c++", os.path.join(ROOT, "tests", "fake_engine", "fake_engine.cpp"), "-o", out]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    lib = L.bind(C.CDLL(out))
    lib.fake_ctx_create.argtypes = [C.c_int64, L.P_f64, L.P_f64, C.c_double, C.POINTER(C.c_void_p)]
    lib.fake_ctx_destroy.argtypes = [C.c_void_p]
    lib.fake_ctx_destroy.restype = None
    lib.fake_columns_in_use.argtypes = [C.c_void_p]
    lib.fake_columns_in_use.restype = C.c_int64
    lib.fake_requests.argtypes = [C.c_void_p]
    lib.fake_requests.restype = C.c_int64
    lib.fake_slot_stats.argtypes = [C.c_void_p, C.POINTER(C.c_int64)]
    lib.fake_slot_stats.restype = None
    return lib


class FakeCtx:
    """What NativeFits needs of a context: the handle and the last error."""

    def __init__(self, lib, K, diag, step_ms):
        self._lib = lib
        self._h = C.c_void_p()
        K = np.ascontiguousarray(K, np.float64)
        diag = np.ascontiguousarray(diag, np.float64)
        assert lib.fake_ctx_create(K.shape[0], K.ctypes.data_as(L.P_f64), diag.ctypes.data_as(L.P_f64),
                                   float(step_ms), C.byref(self._h)) == 0

    def last_error(self):
        return (self._lib.sg_last_error(self._h) or b"").decode()

    def columns_in_use(self):
        return self._lib.fake_columns_in_use(self._h)

    def requests(self):
        return self._lib.fake_requests(self._h)

    def slot_stats(self):
        """(subset preparations, highest slot prepared or set, most slots with requests at a launch)"""
        out = (C.c_int64 * 3)()
        self._lib.fake_slot_stats(self._h, out)
        return tuple(out)

    def close(self):
        if self._h:
            self._lib.fake_ctx_destroy(self._h)
            self._h = None


@pytest.fixture(scope="module")
def cohort():
    n, m = 200, 500
    bed, _ = synth.synth_bed(77, n, m, 0.02)
    g = plink.setgeno(bed, n, m, np.arange(1, n + 1), np.ones(n, bool), 0.01, 0.15)
    grm = aireml.DenseGRM(g)
    gv = synth.genetic_value_from_codes(g.codes, 9)
    rng = np.random.default_rng(4)
    specs, refs = [], []
    for k, trait in enumerate(["binary", "quantitative", "binary", "quantitative", "binary", "quantitative"]):
        y, Cv = synth.simulate_pheno(gv, 60 + k, trait, tau=0.8, prevalence=0.3, h2=0.5)
        mask = None if k < 2 or k > 3 else rng.uniform(size=n) > 0.25
        S = np.arange(n) if mask is None else np.nonzero(mask)[0]
        f0 = prep.make_fit0(y[S], Cv[S], trait, True)
        specs.append(serve.FitSpec(f0, trait, mask=mask, seed=200 + k))
        refs.append(None if mask is not None else
                    (aireml.glmmkin_binary if trait == "binary" else aireml.glmmkin_quantitative)(
                        grm, f0, seed=200 + k))
    return grm, specs, refs


def _ctx(fake_lib, grm, step_ms=0.0):
    return FakeCtx(fake_lib, grm.K, grm.diag_sum / grm.m_qc if not grm.is_diag_one else np.ones(grm.K.shape[0]),
                   step_ms)


def _run(fake_lib, grm, specs, step_ms=0.0, **kw):
    ctx = _ctx(fake_lib, grm, step_ms)
    try:
        res, jobs = native.fit_batch(ctx, specs, lib=fake_lib, **kw)
        assert ctx.requests() == 0 and ctx.columns_in_use() == 0  # every column consumed or cancelled
    finally:
        ctx.close()
    return res, jobs


def test_native_driver_matches_oracle(fake_lib, cohort):
    """Worker threads resuming fits while the calling thread steps: tau, coefficients and linear
    predictors of the unmasked fits equal the oracle's (same algorithm, same probes, FP64)."""
    grm, specs, refs = cohort
    res, jobs = _run(fake_lib, grm, specs, threads=4)
    for r, ref in zip(res, refs):
        assert not isinstance(r, Exception), r
        if ref is None:
            continue
        np.testing.assert_allclose(r["theta"], ref["theta"], rtol=1e-8)
        np.testing.assert_allclose(r["coefficients"], ref["coefficients"], rtol=1e-8, atol=1e-12)
        np.testing.assert_allclose(r["linear_predictors"], ref["linear_predictors"], rtol=1e-8, atol=1e-12)
        assert r["iterations"] == ref["iterations"]
    assert all(j.column_iterations > 0 for j in jobs)


@pytest.mark.parametrize("mode", [dict(threads=1), dict(threads=4, pipelined=False), dict(threads=3, step_ms=0.3),
                                  dict(threads=4, step_ms=0.3, launch_wait_ms=2.0)])
def test_native_driver_schedules_agree(fake_lib, cohort, mode):
    """The calling thread alone, blocking steps with workers, workers under an emulated step time,
    and launches that wait for the workers give bit-identical fits to the default schedule: a fit's
    columns never depend on what shared their steps."""
    grm, specs, _ = cohort
    base, bj = _run(fake_lib, grm, specs, threads=4)
    mode = dict(mode)
    step_ms = mode.pop("step_ms", 0.0)
    other, oj = _run(fake_lib, grm, specs, step_ms=step_ms, **mode)
    for a, b, ja, jb in zip(base, other, bj, oj):
        assert not isinstance(b, Exception), b
        assert np.array_equal(a["theta"], b["theta"])
        assert np.array_equal(a["coefficients"], b["coefficients"])
        assert np.array_equal(a["linear_predictors"], b["linear_predictors"])
        assert a["iterations"] == b["iterations"] and ja.column_iterations == jb.column_iterations


def test_native_driver_queues_fits_beyond_slots(fake_lib, cohort):
    """More fits than slots: they wait in the queue and take slots as fits finish (probe caches
    cleared between tenants), with the same results as run alone.  The next queued fit holds the
    one spare slot (one per eight fits) and its subset is prepared there while it waits; no more
    than max_phenos fits have columns at once."""
    grm, specs, _ = cohort
    many = [specs[i % len(specs)] for i in range(10)]
    ctx = _ctx(fake_lib, grm, 0.1)
    try:
        res, _ = native.fit_batch(ctx, many, lib=fake_lib, threads=4, max_phenos=3)
        prepares, max_slot, busy = ctx.slot_stats()
    finally:
        ctx.close()
    assert prepares >= len(many) and max_slot == 3 and busy <= 3, (prepares, max_slot, busy)
    alone, _ = _run(fake_lib, grm, specs, threads=1)
    for i, r in enumerate(res):
        assert not isinstance(r, Exception), r
        assert np.array_equal(r["theta"], alone[i % len(specs)]["theta"])


def test_native_driver_failing_fit_and_serving(fake_lib, cohort):
    """A quantitative phenotype with variance << 1 fails with its own error while the others
    finish; arrivals submitted between steps are admitted and all complete."""
    grm, specs, _ = cohort
    n = grm.K.shape[0]
    Cv = np.random.default_rng(5).standard_normal((n, 2))
    bad = serve.FitSpec(prep.make_fit0(0.3 + 1e-4 * np.arange(n) / n, Cv, "quantitative", True), "quantitative")
    res, _ = _run(fake_lib, grm, [specs[0], bad, specs[1]], threads=4)
    assert isinstance(res[1], Exception) and "variance" in str(res[1])
    assert not isinstance(res[0], Exception) and not isinstance(res[2], Exception)
    ctx = _ctx(fake_lib, grm, 0.2)
    try:
        arrivals = [(0.002 * i, specs[i % len(specs)]) for i in range(7)]
        done = native.serve(ctx, arrivals, max_columns=256, max_phenos=2, threads=3, lib=fake_lib)
        assert ctx.requests() == 0
    finally:
        ctx.close()
    assert len(done) == 7 and all(j.error is None for j in done)


@pytest.mark.parametrize("rep", range(3))
def test_native_driver_serving_stress(fake_lib, cohort, rep):
    """Many short arrivals into few slots, with steps of 50 us: fits start, submit and finish while
    the calling thread steps, so every ordering of a worker's submission against a launch and a
    stall check occurs; every fit completes with its result alone."""
    grm, specs, _ = cohort
    alone, _ = _run(fake_lib, grm, specs, threads=1)
    ctx = _ctx(fake_lib, grm, 0.05)
    try:
        arrivals = [(0.0005 * i, specs[(i + rep) % len(specs)]) for i in range(18)]
        done = native.serve(ctx, arrivals, max_columns=256, max_phenos=3, threads=4, lib=fake_lib)
        assert ctx.requests() == 0
    finally:
        ctx.close()
    assert len(done) == 18 and all(j.error is None for j in done)
    for j in done:
        k = specs.index(j.spec)
        assert np.array_equal(j.result["theta"], alone[k]["theta"])
