"""Failure detection without faulting the GPU: bounded device waits, host-side refusals and
per-request failures that leave the other requests running."""
import numpy as np
import pytest

from saigegpu import GRM_FP32_SIMT, MV_FP32_SIMT, Context, SaigeGpuError, prep, serve, synth

pytestmark = pytest.mark.gpu


def test_bounded_device_wait_reports_timeout_and_context_survives():
    with Context(0) as ctx:
        with pytest.raises(SaigeGpuError) as ei:
            ctx._call("sg_selftest_wait_timeout", 50.0)
        assert ei.value.code == 8  # SG_ERR_TIMEOUT
        n, m = 128, 200
        bed, _ = synth.synth_bed(2, n, m, 0.0)
        ctx.setgeno(bed, n, m)  # the context is still usable
        ctx.grm_build(GRM_FP32_SIMT)
        x, it = ctx.pcg_solve(np.full(n, 0.2), np.array([1.0, 0.3]), np.ones(n), 50, 1e-8)
        assert np.isfinite(x).all() and it > 0


def test_hbm_budget_refusal():
    n, m = 4000, 3000
    bed, _ = synth.synth_bed(3, n, m, 0.0)
    with Context(0, hbm_budget_bytes=8 << 20) as ctx:
        with pytest.raises(SaigeGpuError) as ei:
            ctx.setgeno(bed, n, m)
            ctx.grm_build(GRM_FP32_SIMT)
        assert ei.value.code == 3  # SG_ERR_NOMEM


def test_nan_inputs_are_rejected():
    n, m = 256, 300
    bed, _ = synth.synth_bed(4, n, m, 0.0)
    with Context(0) as ctx:
        ctx.setgeno(bed, n, m)
        ctx.grm_build(GRM_FP32_SIMT)
        w = np.full(n, 0.2)
        b = np.ones(n)
        b[7] = np.nan
        with pytest.raises(SaigeGpuError) as ei:
            ctx.pcg_solve(w, np.array([1.0, 0.3]), b)
        assert ei.value.code == 6
        w[3] = np.nan
        with pytest.raises(SaigeGpuError):
            ctx.engine_set_pheno(0, w, np.array([1.0, 0.3]))


def test_failing_and_cancelled_fits_do_not_stop_the_others():
    n, m = 500, 900
    bed, codes = synth.synth_bed(5, n, m, 0.01)
    with Context(0) as ctx:
        ctx.set_matvec_mode(MV_FP32_SIMT)
        ctx.setgeno(bed, n, m)
        ctx.grm_build(GRM_FP32_SIMT)
        gv = synth.genetic_value_from_codes(codes, 2)
        good = []
        for k in range(3):
            y, C = synth.simulate_pheno(gv, 20 + k, "binary", tau=0.5, prevalence=0.3)
            good.append(serve.FitSpec(prep.make_fit0(y, C, "binary", True), "binary"))
        yq = np.random.default_rng(0).standard_normal(n) * 0.01  # var(Y) < 0.1: the fit must stop
        bad = serve.FitSpec(prep.make_fit0(yq, None, "quantitative", False), "quantitative")
        r = serve.Runner(ctx, 512, 4)
        ids = [r.submit(s) for s in good[:2]] + [r.submit(bad), r.submit(good[2])]
        r.step()
        r.cancel(ids[1])
        r.run()
        by = {j.jid: j for j in r.finished}
        assert isinstance(by[ids[2]].error, ValueError)
        assert str(by[ids[1]].error) == "cancelled"
        for i in (ids[0], ids[3]):
            assert by[i].error is None and by[i].result["converged"]
