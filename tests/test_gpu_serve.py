"""Batched multi-phenotype fits on the GPU engine: oracle parity and alone-vs-in-the-mix identity."""
import numpy as np
import pytest

from oracle import aireml, plink
from saigegpu import GRM_FP32_SIMT, MV_BF16X3_TC, MV_FP32_SIMT, MV_TF32X3_TC, prep, serve, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cohort(gpu_ctx):
    n, m = 640, 1600
    bed, _ = synth.synth_bed(41, n, m, 0.02)
    gpu_ctx.set_matvec_mode(MV_FP32_SIMT)
    gpu_ctx.setgeno(bed, n, m)
    gpu_ctx.grm_build(GRM_FP32_SIMT)
    g = plink.setgeno(bed, n, m, np.arange(1, n + 1), np.ones(n, bool), 0.01, 0.15)
    grm = aireml.DenseGRM(g)
    gv = synth.genetic_value_from_codes(g.codes, 7)
    rng = np.random.default_rng(3)
    specs, refs = [], []
    for k, trait in enumerate(["binary", "quantitative", "binary", "quantitative"]):
        y, C = synth.simulate_pheno(gv, 50 + k, trait, tau=0.6, prevalence=0.25, h2=0.5)
        mask = None if k < 2 else rng.uniform(size=n) > 0.2
        S = np.arange(n) if mask is None else np.nonzero(mask)[0]
        f0 = prep.make_fit0(y[S], C[S], trait, True)
        specs.append(serve.FitSpec(f0, trait, mask=mask))
        sub = aireml.DenseGRM.from_matrix(grm.K[np.ix_(S, S)], grm.m_qc, grm.diag_sum[S])
        refs.append((aireml.glmmkin_binary if trait == "binary" else aireml.glmmkin_quantitative)(sub, f0)
                    if mask is None else None)
    return gpu_ctx, grm, specs, refs


def test_batched_fits_match_oracle(cohort):
    ctx, grm, specs, refs = cohort
    res, jobs = serve.fit_batch(ctx, specs, max_columns=256)
    for r, ref in zip(res, refs):
        assert not isinstance(r, Exception), r
        if ref is not None:
            # tau within 1e-4 relative of the FP64 oracle with the same probes
            np.testing.assert_allclose(r["theta"], ref["theta"], rtol=1e-4)
            np.testing.assert_allclose(r["coefficients"], ref["coefficients"], rtol=1e-4, atol=1e-8)


def test_alone_equals_in_the_mix(cohort):
    ctx, grm, specs, refs = cohort
    mix, _ = serve.fit_batch(ctx, specs, max_columns=256)
    for k in (1, 2):
        alone, _ = serve.fit_batch(ctx, [specs[k]], max_columns=256)
        np.testing.assert_allclose(alone[0]["theta"], mix[k]["theta"], rtol=1e-12)
        np.testing.assert_allclose(alone[0]["linear_predictors"], mix[k]["linear_predictors"], rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("mode", [MV_TF32X3_TC, MV_BF16X3_TC])
def test_split_engine_matches_oracle(cohort, mode):
    ctx, grm, specs, refs = cohort
    ctx.set_matvec_mode(mode)
    try:
        res, _ = serve.fit_batch(ctx, specs[:2], max_columns=256)
        for r, ref in zip(res, refs[:2]):
            np.testing.assert_allclose(r["theta"], ref["theta"], rtol=1e-4)
    finally:
        ctx.set_matvec_mode(MV_FP32_SIMT)


def test_serving_stream(cohort):
    ctx, grm, specs, refs = cohort
    arrivals = [(0.02 * i, specs[i % len(specs)]) for i in range(6)]
    done = serve.serve(ctx, arrivals, max_columns=128, max_phenos=3)
    assert len(done) == 6
    assert all(j.error is None for j in done)
    lat = [j.t_done - j.t_arrive for j in done]
    assert min(lat) > 0


@pytest.mark.parametrize("mode", [MV_FP32_SIMT, MV_TF32X3_TC, MV_BF16X3_TC])
def test_pipelined_runner_equals_synchronous(cohort, mode):
    """Launch/finish stepping (host consumes step k while step k+1 runs) changes when columns
    start, not what they compute: every fit is bit-identical to the blocking runner's."""
    ctx, grm, specs, refs = cohort
    ctx.set_matvec_mode(mode)
    try:
        sync, _ = serve.fit_batch(ctx, specs, max_columns=256, pipelined=False)
        pipe, _ = serve.fit_batch(ctx, specs, max_columns=256, pipelined=True)
    finally:
        ctx.set_matvec_mode(MV_FP32_SIMT)
    for a, b in zip(pipe, sync):
        assert not isinstance(a, Exception), a
        np.testing.assert_array_equal(a["theta"], b["theta"])
        np.testing.assert_array_equal(a["coefficients"], b["coefficients"])
        np.testing.assert_array_equal(a["linear_predictors"], b["linear_predictors"])


def test_launch_finish_with_host_calls_in_flight(cohort):
    """Fetch, cancel, submit and weight uploads of an idle slot while a step runs."""
    ctx, grm, specs, refs = cohort
    n = ctx.n
    rng = np.random.default_rng(11)
    w = rng.uniform(0.5, 2.0, n)
    tau = np.array([1.0, 0.4])
    B = rng.standard_normal((n, 6))
    ctx.engine_reserve(128, 2)
    ctx.engine_hold_results(True)
    try:
        ctx.engine_set_pheno(0, w, tau)
        ids = ctx.engine_submit(0, 0, B[:, :3], 500, 1e-10)
        launched, _ = ctx.engine_launch()
        assert launched
        with pytest.raises(Exception):
            ctx.engine_launch()  # one step in flight at a time
        ctx.engine_set_pheno(1, w * 1.5, tau)  # slot 1 has no columns: allowed in flight
        more = ctx.engine_submit(1, 0, B[:, 3:5], 500, 1e-10)  # joins the next launch
        ctx.engine_cancel(int(more[1]))
        done = {}
        for _ in range(2000):  # every column stops within maxiter = 500 steps
            if len(done) == 4:
                break
            ctx.engine_finish()
            for rid in ctx.engine_poll():
                done[int(rid)] = ctx.engine_fetch(int(rid))[0]
            ctx.engine_launch()
        ctx.engine_finish()
        assert set(done) == set(int(i) for i in ids) | {int(more[0])}
        # the same solves through the blocking path
        ctx.engine_hold_results(False)
        ids2 = ctx.engine_submit(0, 0, B[:, :3], 500, 1e-10)
        ids3 = ctx.engine_submit(1, 0, B[:, 3:4], 500, 1e-10)
        got = {}
        for _ in range(2000):
            if len(got) == 4:
                break
            ctx.engine_run(1)
            for rid in ctx.engine_poll():
                got[int(rid)] = ctx.engine_fetch(int(rid))[0]
        for a, b in zip(list(ids) + [more[0]], list(ids2) + [ids3[0]]):
            np.testing.assert_array_equal(done[int(a)], got[int(b)])
    finally:
        ctx.engine_hold_results(False)


def test_exact_subset_fits_match_oracle_on_subset_cohort():
    """Per-subset exactness: allele frequencies, QC and K recomputed on the phenotype's samples,
    like the reference's setgeno with that sample list; the oracle does the same on the CPU."""
    from saigegpu import Context
    n, m = 520, 1400
    bed, _ = synth.synth_bed(61, n, m, 0.02)
    gpu_ctx = Context(0)
    gpu_ctx.setgeno(bed, n, m)
    gpu_ctx.grm_build(GRM_FP32_SIMT)
    gpu_ctx.set_matvec_mode(MV_FP32_SIMT)
    g_all = plink.setgeno(bed, n, m, np.arange(1, n + 1), np.ones(n, bool), 0.01, 0.15)
    gv = synth.genetic_value_from_codes(g_all.codes, 9)
    rng = np.random.default_rng(8)
    specs, refs = [], []
    for k, trait in enumerate(["binary", "quantitative"]):
        mask = rng.uniform(size=n) > 0.3
        S = np.nonzero(mask)[0]
        y, C = synth.simulate_pheno(gv, 70 + k, trait, tau=0.6, prevalence=0.3, h2=0.5)
        f0 = prep.make_fit0(y[S], C[S], trait, True)
        specs.append(serve.FitSpec(f0, trait, mask=mask))
        g_sub = plink.setgeno(bed, n, m, S + 1, mask, 0.01, 0.15)
        sub = aireml.DenseGRM(g_sub)
        refs.append((aireml.glmmkin_binary if trait == "binary" else aireml.glmmkin_quantitative)(sub, f0))
    before = gpu_ctx.dims()
    res, _ = serve.fit_batch_exact_subsets(gpu_ctx, specs, max_columns=256)
    assert gpu_ctx.dims() == before  # the full cohort is restored
    for r, ref in zip(res, refs):
        assert not isinstance(r, Exception), r
        np.testing.assert_allclose(r["theta"], ref["theta"], rtol=1e-4)
        np.testing.assert_allclose(r["coefficients"], ref["coefficients"], rtol=1e-4, atol=1e-8)
    gpu_ctx.close()


@pytest.mark.parametrize("mode", [MV_FP32_SIMT, MV_BF16X3_TC])
def test_native_driver_matches_python_driver_and_oracle(cohort, mode):
    """The C++ fit driver (sg_fits_*) runs the same algorithm as the Python generators: the same
    iterations, tau to rounding, and the oracle's tau to 1e-4 (masked fits included)."""
    from saigegpu import native
    ctx, grm, specs, refs = cohort
    ctx.set_matvec_mode(mode)
    try:
        py, _ = serve.fit_batch(ctx, specs, max_columns=256)
        nat, jobs = native.fit_batch(ctx, specs, max_columns=256)
    finally:
        ctx.set_matvec_mode(MV_FP32_SIMT)
    for a, b, ref, j in zip(nat, py, refs, jobs):
        assert not isinstance(a, Exception), a
        assert a["iterations"] == b["iterations"]
        np.testing.assert_allclose(a["theta"], b["theta"], rtol=1e-8)
        np.testing.assert_allclose(a["coefficients"], b["coefficients"], rtol=1e-7, atol=1e-10)
        np.testing.assert_allclose(a["linear_predictors"], b["linear_predictors"], rtol=1e-7, atol=1e-10)
        assert j.column_iterations > 0
        if ref is not None:
            np.testing.assert_allclose(a["theta"], ref["theta"], rtol=1e-4)


def test_native_driver_failing_fit_and_serving(cohort):
    """A fit that fails (quantitative phenotype with variance << 1) reports its own error; the
    others finish; served arrivals all complete."""
    from saigegpu import native
    ctx, grm, specs, refs = cohort
    n = ctx.n
    C = np.random.default_rng(5).standard_normal((n, 2))
    y_flat = 0.3 + 1e-4 * np.arange(n) / n
    bad = serve.FitSpec(prep.make_fit0(y_flat, C, "quantitative", True), "quantitative")
    res, _ = native.fit_batch(ctx, [specs[0], bad, specs[1]], max_columns=256)
    assert isinstance(res[1], Exception) and "variance" in str(res[1])
    assert not isinstance(res[0], Exception) and not isinstance(res[2], Exception)
    arrivals = [(0.01 * i, specs[i % len(specs)]) for i in range(5)]
    done = native.serve(ctx, arrivals, max_columns=256, max_phenos=2)
    assert len(done) == 5 and all(j.error is None for j in done)


def test_chained_solve_equals_solve_of_fetched_product(cohort):
    """A solve chained to a product (Sigma x = K b on the engine) equals the solve of the fetched
    product bit for bit: admitted after the product finished, after the product was fetched first
    (its result handed to the solve's own right-hand side), and cancelled with an unfinished source."""
    from saigegpu import _lib as L
    ctx, grm, specs, refs = cohort
    n = ctx.n
    rng = np.random.default_rng(21)
    w = rng.uniform(0.5, 2.0, n)
    tau = np.array([1.0, 0.4])
    b = rng.standard_normal((n, 3))
    ctx.engine_reserve(128, 2)
    ctx.engine_hold_results(True)

    def drive(want):
        done = set()
        for _ in range(3000):
            if want <= done:
                return
            ctx.engine_launch()
            ctx.engine_finish()
            done.update(int(r) for r in ctx.engine_poll())
        raise AssertionError("engine did not finish %s" % sorted(want - done))

    def solve_direct(rhs):
        d = int(ctx.engine_submit(0, 0, rhs, 500, 1e-10)[0])
        drive({d})
        return ctx.engine_fetch(d)[0]

    try:
        ctx.engine_set_pheno(0, w, tau)
        # admitted once the product is done
        p0 = int(ctx.engine_submit(0, 1, b[:, 0], 1, 0.0)[0])
        c0 = int(ctx.engine_submit_chained(0, [p0], 500, 1e-10)[0])
        drive({p0, c0})
        x0, it0 = ctx.engine_fetch(c0)
        kb0 = ctx.engine_fetch(p0)[0]
        assert it0 > 0
        np.testing.assert_array_equal(x0, solve_direct(kb0))
        # the product fetched before the chained solve was admitted
        p1 = int(ctx.engine_submit(0, 1, b[:, 1], 1, 0.0)[0])
        c1 = int(ctx.engine_submit_chained(0, [p1], 500, 1e-10)[0])
        drive({p1})
        kb1 = ctx.engine_fetch(p1)[0]
        drive({c1})
        np.testing.assert_array_equal(ctx.engine_fetch(c1)[0], solve_direct(kb1))
        # a source cancelled before it ran takes its chained solve with it
        p2 = int(ctx.engine_submit(0, 1, b[:, 2], 1, 0.0)[0])
        c2 = int(ctx.engine_submit_chained(0, [p2], 500, 1e-10)[0])
        ctx.engine_cancel(p2)
        with pytest.raises(L.SaigeGpuError):
            ctx.engine_fetch(c2)
        launched, _ = ctx.engine_launch()
        assert not launched
    finally:
        ctx.engine_hold_results(False)


def test_launch_finish_retires_columns_that_converge_at_init(cohort):
    """With asynchronous stepping a zero right-hand side (r'r = 0 at init) is retired when the step
    it rode along finishes: zero iterations, zero solution; the other columns are unaffected."""
    ctx, grm, specs, refs = cohort
    n = ctx.n
    rng = np.random.default_rng(12)
    w = rng.uniform(0.5, 2.0, n)
    tau = np.array([1.0, 0.4])
    B = rng.standard_normal((n, 3))
    B[:, 1] = 0.0
    ctx.engine_reserve(128, 2)
    ctx.engine_hold_results(True)
    try:
        ctx.engine_set_pheno(0, w, tau)
        ids = [int(i) for i in ctx.engine_submit(0, 0, B, 500, 1e-10)]
        got = {}
        for _ in range(2000):
            if len(got) == 3:
                break
            ctx.engine_launch()
            ctx.engine_finish()
            for rid in ctx.engine_poll():
                got[int(rid)] = ctx.engine_fetch(int(rid))
        assert set(got) == set(ids)
        x0, it0 = got[ids[1]]
        assert it0 == 0 and not np.any(x0)
        ctx.engine_hold_results(False)
        ref = {}
        ids2 = [int(i) for i in ctx.engine_submit(0, 0, B[:, [0, 2]], 500, 1e-10)]
        for _ in range(2000):
            if len(ref) == 2:
                break
            ctx.engine_run(1)
            for rid in ctx.engine_poll():
                ref[int(rid)] = ctx.engine_fetch(int(rid))[0]
        np.testing.assert_array_equal(got[ids[0]][0], ref[ids2[0]])
        np.testing.assert_array_equal(got[ids[2]][0], ref[ids2[1]])
    finally:
        ctx.engine_hold_results(False)


def test_native_fit_with_many_covariates_matches_oracle(cohort):
    """Seven design columns (covariates not folded into the offset): the probe reductions carry
    2 + 2 p = 16 sums per probe, past the kernel's four-covariate fast path."""
    from saigegpu import native
    ctx, grm, specs, refs = cohort
    n = grm.n
    rng = np.random.default_rng(17)
    gv = synth.genetic_value_from_codes(plink.setgeno(*_cohort_bed(), np.arange(1, n + 1), np.ones(n, bool),
                                                      0.01, 0.15).codes, 11)
    y, C = synth.simulate_pheno(gv, 91, "binary", tau=0.6, prevalence=0.3, h2=0.5)
    C6 = np.column_stack([C, rng.standard_normal((n, 4))])
    f0 = prep.make_fit0(y, C6, "binary", False)
    assert f0["X"].shape[1] == 7
    ref = aireml.glmmkin_binary(grm, f0)
    res, _ = native.fit_batch(ctx, [serve.FitSpec(f0, "binary")], max_columns=256)
    assert not isinstance(res[0], Exception), res[0]
    np.testing.assert_allclose(res[0]["theta"], ref["theta"], rtol=1e-4)


def _cohort_bed():
    n, m = 640, 1600
    bed, _ = synth.synth_bed(41, n, m, 0.02)
    return bed, n, m
