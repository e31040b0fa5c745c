"""Host logic of the batched driver, run against a numpy fake of the engine (no GPU)."""
import numpy as np

from oracle import aireml, plink, probes
from saigegpu import prep, serve, synth


class FakeEngine:
    """Implements the engine calls the runner uses with the FP64 oracle (solves on admission)."""

    def __init__(self, grm):
        self.cache = {}
        self.grm = grm
        self.n = grm.n
        self.ph = {}
        self.res = {}
        self.fin = []
        self.next = 1

    def engine_reserve(self, cols, phenos):
        pass

    def engine_set_pheno(self, slot, w, tau, mask=None):
        self.ph[slot] = (np.asarray(w, float).copy(), np.asarray(tau, float).copy(),
                         np.ones(self.n, bool) if mask is None else np.asarray(mask, bool))

    def _solve(self, slot, kind, b, maxiter, tol):
        w, tau, m = self.ph[slot]
        S = np.nonzero(m)[0]
        b = np.where(m, b, 0.0)
        x = np.zeros(self.n)
        if kind == 1:
            x[S] = self.grm.K[np.ix_(S, S)] @ b[S]
            return x, 1
        sub = aireml.DenseGRM.from_matrix(self.grm.K[np.ix_(S, S)], self.grm.m_qc, self.grm.diag_sum[S])
        xs, it = aireml.pcg(sub, w[S], tau, b[S], maxiter, tol, return_iters=True)
        x[S] = xs
        return x, int(np.asarray(it).ravel()[0])

    def engine_submit(self, slot, kind, B, maxiter=500, tol=1e-5):
        B = np.asarray(B, float)
        ids = []
        for j in range(B.shape[1]):
            rid = self.next
            self.next += 1
            self.res[rid] = self._solve(slot, kind, B[:, j], maxiter, tol)
            self.fin.append(rid)
            ids.append(rid)
        return np.array(ids)

    def engine_submit_probes(self, slot, kind, seed, run0, k, maxiter=500, tol=1e-5):
        U = np.column_stack([probes.rademacher(seed, run0 + j, self.n) for j in range(k)])
        return self.engine_submit(slot, kind, U, maxiter, tol)

    def engine_run(self, k=1):
        return len(self.fin)

    def engine_poll(self, max_ids=1 << 16):
        out, self.fin = self.fin, []
        return np.array(out, dtype=np.int64)

    def engine_fetch(self, rid):
        return self.res.pop(int(rid))

    def engine_probe_cached(self, slot, seed, run):
        return (slot, seed, run) in self.cache

    def engine_probe_cache_clear(self, slot=-1):
        self.cache = {k: v for k, v in getattr(self, "cache", {}).items() if slot >= 0 and k[0] != slot}

    def engine_probe_dots(self, slot, pid, aid, seed, run0, SX):
        m = self.ph[slot][2]
        self.cache = getattr(self, "cache", {})
        rows, its = [], []
        for j, (a, b) in enumerate(zip(pid, aid)):
            su, it = self.res.pop(int(a))
            if int(b) < 0:
                au = self.cache[(slot, seed, run0 + j)]
            else:
                au, _ = self.res.pop(int(b))
                self.cache[(slot, seed, run0 + j)] = au
            u = probes.rademacher(seed, run0 + j, self.n) * m
            rows.append(np.concatenate([[au @ su, u @ su], au @ SX, SX.T @ u]))
            its.append(it)
        return np.array(rows), np.array(its)

    def engine_cancel(self, rid):
        self.res.pop(int(rid), None)


def _cohort(seed=13, n=240, m=700):
    bed, _ = synth.synth_bed(seed, n, m, 0.01)
    g = plink.setgeno(bed, n, m, np.arange(1, n + 1), np.ones(n, bool), 0.01, 0.15)
    return aireml.DenseGRM(g), g


def test_generator_fit_equals_oracle_fit():
    grm, g = _cohort()
    n = grm.n
    gv = synth.genetic_value_from_codes(g.codes, 3)
    for trait in ("binary", "quantitative"):
        y, C = synth.simulate_pheno(gv, 5, trait, tau=0.5, prevalence=0.3, h2=0.5)
        f0 = prep.make_fit0(y, C, trait, True)
        ref = (aireml.glmmkin_binary if trait == "binary" else aireml.glmmkin_quantitative)(grm, f0)
        res, jobs = serve.fit_batch(FakeEngine(grm), [serve.FitSpec(f0, trait)])
        # same algorithm in FP64; only the summation order differs
        np.testing.assert_allclose(res[0]["theta"], ref["theta"], rtol=1e-9)
        np.testing.assert_allclose(res[0]["coefficients"], ref["coefficients"], rtol=1e-9, atol=1e-12)
        assert res[0]["iterations"] == ref["iterations"]


def test_masked_fit_equals_subset_fit():
    grm, g = _cohort(17)
    n = grm.n
    rng = np.random.default_rng(2)
    mask = rng.uniform(size=n) > 0.25
    S = np.nonzero(mask)[0]
    gv = synth.genetic_value_from_codes(g.codes, 4)
    y, C = synth.simulate_pheno(gv, 6, "binary", tau=0.5, prevalence=0.3)
    f0 = prep.make_fit0(y[S], C[S], "binary", True)
    sub = aireml.DenseGRM.from_matrix(grm.K[np.ix_(S, S)], grm.m_qc, grm.diag_sum[S])
    ref = aireml.glmmkin_binary(sub, f0)
    # probes over the subset: the driver masks cohort-length probes, so draw the oracle's the same way
    res, _ = serve.fit_batch(FakeEngine(grm), [serve.FitSpec(f0, "binary", mask=mask)])
    assert res[0]["n"] == len(S)
    assert abs(res[0]["theta"][1] - ref["theta"][1]) / ref["theta"][1] < 0.2


class FakeAsyncEngine(FakeEngine):
    """FakeEngine with the launch/finish protocol: work submitted before a launch completes at
    the matching finish, so results reach the driver one step late as in the pipelined engine."""

    def __init__(self, grm):
        super().__init__(grm)
        self.queued, self.running = [], []
        self.launches = 0

    def engine_submit(self, slot, kind, B, maxiter=500, tol=1e-5):
        ids = super().engine_submit(slot, kind, B, maxiter, tol)
        done = set(int(i) for i in ids)
        self.fin = [i for i in self.fin if i not in done]
        self.queued += [int(i) for i in ids]
        return ids

    def engine_run(self, k=1):
        raise AssertionError("the pipelined runner must not call engine_run")

    def engine_launch(self):
        if self.running:
            raise RuntimeError("a step is in flight")
        self.running, self.queued = self.queued, []
        self.launches += bool(self.running)
        return bool(self.running), 0

    def engine_finish(self):
        n = len(self.running)
        self.fin += self.running
        self.running = []
        return n


def test_pipelined_runner_matches_synchronous_runner():
    grm, g = _cohort(19)
    gv = synth.genetic_value_from_codes(g.codes, 5)
    specs = []
    for k, trait in enumerate(("binary", "quantitative", "binary")):
        y, C = synth.simulate_pheno(gv, 20 + k, trait, tau=0.5, prevalence=0.3, h2=0.5)
        specs.append(serve.FitSpec(prep.make_fit0(y, C, trait, True), trait))
    ref, _ = serve.fit_batch(FakeEngine(grm), specs)
    eng = FakeAsyncEngine(grm)
    res, jobs = serve.fit_batch(eng, specs, pipelined=True)
    assert eng.launches > 0 and not eng.running and not eng.queued
    for a, b in zip(res, ref):
        assert not isinstance(a, Exception), a
        np.testing.assert_array_equal(a["theta"], b["theta"])
        np.testing.assert_array_equal(a["coefficients"], b["coefficients"])
        assert a["iterations"] == b["iterations"]


def test_pipelined_runner_with_a_tiny_host_budget():
    """A GPU step that takes no time leaves the host a budget of one fit per step: the deferred
    fits resume on later steps and every result is unchanged."""
    grm, g = _cohort(29)
    gv = synth.genetic_value_from_codes(g.codes, 8)
    specs = []
    for k, trait in enumerate(("binary", "quantitative", "binary", "quantitative")):
        y, C = synth.simulate_pheno(gv, 40 + k, trait, tau=0.5, prevalence=0.3, h2=0.5)
        specs.append(serve.FitSpec(prep.make_fit0(y, C, trait, True), trait))
    ref, _ = serve.fit_batch(FakeEngine(grm), specs)

    class Timed(FakeAsyncEngine):
        ms = 0.0

        def engine_finish(self):
            self.ms += 1e-9
            return super().engine_finish()

        def engine_timing(self):
            return {"step_ms": self.ms}

    eng = Timed(grm)
    res, _ = serve.fit_batch(eng, specs, pipelined=True)
    for a, b in zip(res, ref):
        assert not isinstance(a, Exception), a
        np.testing.assert_array_equal(a["theta"], b["theta"])


def test_pipelined_runner_reports_a_stall():
    grm, g = _cohort(23)
    gv = synth.genetic_value_from_codes(g.codes, 6)
    y, C = synth.simulate_pheno(gv, 31, "quantitative", tau=0.5, h2=0.5)
    spec = serve.FitSpec(prep.make_fit0(y, C, "quantitative", True), "quantitative")

    class Lossy(FakeAsyncEngine):
        def engine_launch(self):  # drops every queued column: nothing ever finishes
            self.queued = []
            return False, 0

    r = serve.Runner(Lossy(grm), 256, 1, pipelined=True)
    r.submit(spec)
    import pytest
    with pytest.raises(RuntimeError, match="engine idle"):
        r.run()


class FakeCohortEngine(FakeEngine):
    """FakeEngine over a cohort that ``set_cohort`` reloads from the bed on the CPU oracle."""

    def __init__(self, bed, n_fam, m_bim):
        self.bed, self.n_fam, self.m_bim = bed, n_fam, m_bim
        self.loads = 0
        self.set_cohort(np.arange(1, n_fam + 1, dtype=np.int32), np.ones(n_fam, np.uint8))

    def cohort(self):
        return dict(sub=self.sub.copy(), mask=self.fmask.copy(), grm=0, mode=0)

    def set_cohort(self, sub_1based, pheno_mask, grm=None, mode=None):
        self.sub, self.fmask = np.asarray(sub_1based, np.int32), np.asarray(pheno_mask, np.uint8)
        g = plink.setgeno(self.bed, self.n_fam, self.m_bim, self.sub, self.fmask.astype(bool), 0.01, 0.15)
        FakeEngine.__init__(self, aireml.DenseGRM(g))
        self.loads += 1

    def dims(self):
        return dict(n=self.n)


def test_exact_subset_grouping_and_restore():
    n, m = 260, 800
    bed, _ = synth.synth_bed(37, n, m, 0.02)
    eng = FakeCohortEngine(bed, n, m)
    g = plink.setgeno(bed, n, m, np.arange(1, n + 1), np.ones(n, bool), 0.01, 0.15)
    gv = synth.genetic_value_from_codes(g.codes, 2)
    rng = np.random.default_rng(4)
    masks = [None, rng.uniform(size=n) > 0.3, None]
    masks.append(masks[1].copy())  # a second fit on the same subset: one rebuild for both
    specs, refs = [], []
    for k, mask in enumerate(masks):
        trait = "quantitative" if k % 2 else "binary"
        S = np.arange(n) if mask is None else np.nonzero(mask)[0]
        y, C = synth.simulate_pheno(gv, 90 + k, trait, tau=0.5, prevalence=0.3, h2=0.5)
        f0 = prep.make_fit0(y[S], C[S], trait, True)
        specs.append(serve.FitSpec(f0, trait, mask=mask))
        gs = plink.setgeno(bed, n, m, S + 1, np.isin(np.arange(n), S), 0.01, 0.15)
        refs.append((aireml.glmmkin_binary if trait == "binary" else aireml.glmmkin_quantitative)(aireml.DenseGRM(gs), f0))
    res, _ = serve.fit_batch_exact_subsets(eng, specs)
    assert eng.loads == 3  # initial load, one subset, the restore
    assert eng.n == n and np.array_equal(eng.sub, np.arange(1, n + 1))
    for r, ref in zip(res, refs):
        assert not isinstance(r, Exception), r
        np.testing.assert_allclose(r["theta"], ref["theta"], rtol=1e-9)


class FakeLocoEngine(FakeEngine):
    """FakeEngine whose loco_set swaps in the oracle's leave-one-chromosome-out GRM."""

    def __init__(self, grm, geno):
        super().__init__(grm)
        self.full, self.geno = grm, geno

    def loco_set(self, begin, end):
        self.grm = aireml.loco_grm(self.full, self.geno, begin, end)

    def loco_clear(self):
        self.grm = self.full

    def loco_set_bim(self, begin, end):
        """A .bim range: the GRM markers inside it (the QC-passing .bim markers, in order)."""
        qc = np.asarray(self.geno.qc_mask, bool)
        b = int(np.count_nonzero(qc[:begin]))
        self.loco_set(b, b + int(np.count_nonzero(qc[begin:end + 1])) - 1)


def test_loco_generator_matches_oracle():
    grm, g = _cohort(43, n=200, m=600)
    gv = synth.genetic_value_from_codes(g.codes, 5)
    chrom = np.repeat(np.arange(1, 23), -(-grm.m_qc // 22))[:grm.m_qc]
    ranges = serve.loco_ranges(chrom)
    for trait in ("binary", "quantitative"):
        y, C = synth.simulate_pheno(gv, 8, trait, tau=0.6, prevalence=0.3, h2=0.5)
        f0 = prep.make_fit0(y, C, trait, True)
        fit = (aireml.glmmkin_binary if trait == "binary" else aireml.glmmkin_quantitative)(grm, f0)
        sel = {c: ranges[c] for c in (3, 17)}
        got = serve.fit_loco(FakeLocoEngine(grm, g), [serve.FitSpec(f0, trait)], [fit], sel)
        for c, (b, e) in sel.items():
            ref = aireml.get_coef_loco(aireml.loco_grm(grm, g, b, e), f0, fit, trait)
            r = got[c][0]
            assert not isinstance(r, Exception), r
            np.testing.assert_allclose(r["coefficients"], ref["alpha"], rtol=1e-9)
            np.testing.assert_allclose(r["linear_predictors"], ref["eta"], rtol=1e-9, atol=1e-12)


def test_loco_with_bim_ranges_equals_grm_ranges():
    """fit_loco over .bim ranges (what the subset-exact engines take) gives the GRM-range results
    when each range holds the same GRM markers."""
    grm, g = _cohort(44, n=180, m=500)
    gv = synth.genetic_value_from_codes(g.codes, 6)
    y, C = synth.simulate_pheno(gv, 9, "binary", tau=0.6, prevalence=0.3)
    f0 = prep.make_fit0(y, C, "binary", True)
    fit = aireml.glmmkin_binary(grm, f0)
    bim_chrom = 1 + (np.arange(len(g.qc_mask)) * 22) // len(g.qc_mask)
    bim_ranges = serve.loco_ranges(bim_chrom)
    grm_ranges = serve.loco_ranges(bim_chrom[np.asarray(g.qc_mask, bool)])
    sel = (5, 19)
    spec = [serve.FitSpec(f0, "binary")]
    by_bim = serve.fit_loco(FakeLocoEngine(grm, g), spec, [fit], {c: bim_ranges[c] for c in sel}, bim=True)
    by_grm = serve.fit_loco(FakeLocoEngine(grm, g), spec, [fit], {c: grm_ranges[c] for c in sel})
    for c in sel:
        np.testing.assert_array_equal(by_bim[c][0]["coefficients"], by_grm[c][0]["coefficients"])
        np.testing.assert_array_equal(by_bim[c][0]["linear_predictors"], by_grm[c][0]["linear_predictors"])
