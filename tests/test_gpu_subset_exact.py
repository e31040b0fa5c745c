"""Subset-exact engine: each phenotype's GRM from its own sample subset, as the reference builds it.

The reference runs setgeno over every phenotype's samples (FIT.cpp:376-385, 436-495), so allele
frequencies, the integer fill, QC and 1/sd are the subset's; the cohort GRM restricted to the
subset (the masked engines) is a different matrix.  Here the subset-exact engine is held to the
FP64 oracle built over the subset (oracle.plink.setgeno with that subset), with the same probes,
and the masked approximation's error is measured against it.
"""
import numpy as np
import pytest

from oracle import aireml, plink
from saigegpu import (MV_FP32_SIMT, MV_SUBSET_EXACT, MV_SUBSET_EXACT_F8, TC_SUBSET_PAIR, TC_SUBSET_SLICE, native,
                      output, prep, serve, synth, vr)

pytestmark = pytest.mark.gpu

N, M = 1800, 4000
DROPS = (0.05, 0.2, 0.4, 0.3)
# BF16 high + low halves, and FP16 high + E4M3 low halves of power-of-two-scaled columns
MODES = [MV_SUBSET_EXACT, MV_SUBSET_EXACT_F8]


def _subset_grm(bed, mask):
    S = np.nonzero(mask)[0]
    g = plink.setgeno(bed, N, M, S + 1, mask, 0.01, 0.15)
    grm = aireml.DenseGRM(g)
    grm.probe_index = S  # the engine hashes the cohort positions of the subset's samples
    return grm


def _run_products(ctx, ids):
    """Steps the engine until every request in ids has finished; returns their results by id."""
    pending = [int(i) for i in ids]
    out = {}
    for _ in range(1000):
        if not pending:
            break
        ctx.engine_run()
        for i in list(pending):
            r = ctx.engine_try_fetch(i)
            if r is not None:
                out[i] = r[0]
                pending.remove(i)
    assert not pending, pending
    return out


@pytest.fixture(scope="module")
def exact_cohort(gpu_ctx):
    bed, _ = synth.synth_bed(77, N, M, 0.02)
    gpu_ctx.set_matvec_mode(MV_FP32_SIMT)
    gpu_ctx.setgeno(bed, N, M)
    g = plink.setgeno(bed, N, M, np.arange(1, N + 1), np.ones(N, bool), 0.01, 0.15)
    gv = synth.genetic_value_from_codes(g.codes, 9)
    gv = gv / gv.std()
    rng = np.random.default_rng(12)
    cases = []
    for k, drop in enumerate(DROPS):
        trait = "binary" if k % 2 == 0 else "quantitative"
        mask = rng.uniform(size=N) > drop
        S = np.nonzero(mask)[0]
        y, C = synth.simulate_pheno(gv, 300 + k, trait, tau=0.5, prevalence=0.25, h2=0.5)
        f0 = prep.make_fit0(y[S], C[S], trait, True)
        cases.append((trait, mask, f0))
    return gpu_ctx, bed, g, cases


@pytest.mark.parametrize("mode", MODES)
def test_subset_exact_products_match_oracle(exact_cohort, mode):
    """Engine products K_S v (kind 1 columns) against the FP64 GRM built over each subset."""
    ctx, bed, _, cases = exact_cohort
    rng = np.random.default_rng(5)
    ctx.set_matvec_mode(mode)
    variants = ((0, 64), (1, 128), (2, 128), (0, 256), (1, 256)) if mode == MV_SUBSET_EXACT else ((0, 256), (1, 256))
    try:
        for pair, sl in variants:
            ctx.set_tc_option(TC_SUBSET_PAIR, pair)
            ctx.set_tc_option(TC_SUBSET_SLICE, sl)
            ctx.engine_reserve(128, len(cases))
            ids = []
            Vs = []
            for slot, (_, mask, _) in enumerate(cases):
                ctx.engine_set_pheno(slot, np.ones(N), np.array([1.0, 0.5]), mask)
                V = rng.standard_normal((N, 7)) + 0.5  # a nonzero mean exercises the centring
                V[~mask] = 0.0
                Vs.append(V)
                ids.append(ctx.engine_submit(slot, 1, V))
            got = _run_products(ctx, np.concatenate(ids))
            for (trait, mask, _), V, idk in zip(cases, Vs, ids):
                S = np.nonzero(mask)[0]
                grm = _subset_grm(bed, mask)
                ref = grm.K @ V[S]
                Y = np.column_stack([got[int(i)] for i in idk])[S]
                err = np.abs(Y - ref).max() / np.abs(ref).max()
                assert err < 6e-5, (pair, trait, err)
    finally:
        ctx.set_tc_option(TC_SUBSET_PAIR, 2)
        ctx.set_tc_option(TC_SUBSET_SLICE, 256)
        ctx.set_matvec_mode(MV_FP32_SIMT)


def test_subset_exact_variants_bit_identical(exact_cohort):
    """CTA pairs and K slices of the genotype GEMMs give the same products, bit for bit, at every
    launch width (one column to wide blocks)."""
    ctx, bed, _, cases = exact_cohort
    rng = np.random.default_rng(6)
    ctx.set_matvec_mode(MV_SUBSET_EXACT)
    try:
        for k in (1, 40, 200, 300):
            V = rng.standard_normal((N, k))
            outs = []
            for pair, sl in ((0, 64), (0, 128), (1, 64), (1, 128), (0, 256), (1, 256), (0, 512), (1, 512)):
                ctx.set_tc_option(TC_SUBSET_PAIR, pair)
                ctx.set_tc_option(TC_SUBSET_SLICE, sl)
                outs.append(ctx.grm_matmul(V))
            for o in outs[1:]:
                np.testing.assert_array_equal(o, outs[0])
            # and through a per-width plan (the tuner's table)
            ctx.set_subset_plan([(64, 0, 256), (192, 0, 128), (1 << 30, 1, 64)])
            np.testing.assert_array_equal(ctx.grm_matmul(V), outs[0])
            ctx.set_subset_plan([])
    finally:
        ctx.set_subset_plan([])
        ctx.set_tc_option(TC_SUBSET_PAIR, 2)
        ctx.set_tc_option(TC_SUBSET_SLICE, 256)
        ctx.set_matvec_mode(MV_FP32_SIMT)


@pytest.mark.parametrize("mode", MODES)
def test_subset_exact_fits_match_oracle_and_masked_error_is_bounded(exact_cohort, mode):
    """Native batched fits on the subset-exact engine: tau within 1e-4 of the FP64 oracle on the
    subset-built GRM (same probes).  The masked approximation (cohort GRM restricted to S) is
    measured against the same exact answer: at this N it is off by percent, far beyond 1e-4."""
    ctx, bed, g, cases = exact_cohort
    specs = [serve.FitSpec(f0, trait, mask=mask) for trait, mask, f0 in cases]
    ctx.set_matvec_mode(mode)
    try:
        res, _ = native.fit_batch(ctx, specs, max_columns=256)
    finally:
        ctx.set_matvec_mode(MV_FP32_SIMT)
    Kc = aireml.DenseGRM(g)
    masked_err = []
    for (trait, mask, f0), r in zip(cases, res):
        assert not isinstance(r, Exception), r
        S = np.nonzero(mask)[0]
        fit = aireml.glmmkin_binary if trait == "binary" else aireml.glmmkin_quantitative
        ref = fit(_subset_grm(bed, mask), f0)
        # BF16 halves: tau within 1e-4 of FP64 (measured 1e-6 to 3e-6 here).  FP16 + E4M3 halves
        # (15 significant bits at a column's top, fewer for entries far below it): measured up to
        # 1.6e-4 on the first binary phenotype, so that form is held to 3e-4 and is not the default
        rel = np.abs(np.asarray(r["theta"]) - ref["theta"]) / np.abs(ref["theta"])
        print("mode %d %s: tau rel error %s" % (mode, trait, rel))
        np.testing.assert_allclose(r["theta"], ref["theta"], rtol=1e-4 if mode == MV_SUBSET_EXACT else 3e-4)
        sub = aireml.DenseGRM.from_matrix(Kc.K[np.ix_(S, S)], Kc.m_qc, Kc.diag_sum[S])
        sub.probe_index = S
        approx = fit(sub, f0)
        masked_err.append(float(np.max(np.abs(approx["theta"] - ref["theta"]) / np.abs(ref["theta"]))))
    # the masked form is an approximation: at N = 1,800 it moved tau by 0.1-6% in the CPU study of
    # this design; it must stay within 10% here and is reported, not claimed exact
    assert max(masked_err) < 0.1, masked_err
    print("masked-vs-exact tau relative error per phenotype:", masked_err)


@pytest.mark.parametrize("mode", MODES)
def test_subset_exact_alone_equals_in_the_mix(exact_cohort, mode):
    ctx, bed, g, cases = exact_cohort
    specs = [serve.FitSpec(f0, trait, mask=mask) for trait, mask, f0 in cases]
    ctx.set_matvec_mode(mode)
    try:
        mix, _ = native.fit_batch(ctx, specs, max_columns=256)
        alone, _ = native.fit_batch(ctx, [specs[2]], max_columns=256)
    finally:
        ctx.set_matvec_mode(MV_FP32_SIMT)
    np.testing.assert_array_equal(alone[0]["theta"], mix[2]["theta"])


@pytest.mark.parametrize("mode", MODES)
def test_subset_exact_full_cohort_matches_cohort_grm(exact_cohort, mode):
    """No mask: the subset is the cohort, and the exact engine's product is the cohort K's."""
    ctx, bed, g, cases = exact_cohort
    grm = aireml.DenseGRM(g)
    V = np.random.default_rng(8).standard_normal((N, 40))
    ctx.set_matvec_mode(mode)
    try:
        Y = ctx.grm_matmul(V)
    finally:
        ctx.set_matvec_mode(MV_FP32_SIMT)
    ref = grm.K @ V
    assert np.abs(Y - ref).max() / np.abs(ref).max() < 6e-5


@pytest.mark.parametrize("mode", MODES)
def test_subset_exact_forget_rebuilds_identically(exact_cohort, mode):
    """Forgetting the kept subset states makes the next set_pheno rebuild them (QC, tables, flip map
    and diagonal on the device); the products after the rebuild are bit-identical."""
    ctx, bed, _, cases = exact_cohort
    rng = np.random.default_rng(9)
    ctx.set_matvec_mode(mode)
    try:
        ctx.engine_reserve(128, len(cases))
        Vs = []
        for _, mask, _ in cases:
            V = rng.standard_normal((N, 5))
            V[~mask] = 0.0
            Vs.append(V)

        def products():
            ids = []
            for slot, (_, mask, _) in enumerate(cases):
                ctx.engine_set_pheno(slot, np.ones(N), np.array([1.0, 0.5]), mask)
                ids.append(ctx.engine_submit(slot, 1, Vs[slot]))
            got = _run_products(ctx, np.concatenate(ids))
            return [np.column_stack([got[int(i)] for i in idk]) for idk in ids]

        first = products()
        ctx.engine_forget_subsets()
        again = products()
        for a, b in zip(first, again):
            np.testing.assert_array_equal(a, b)
    finally:
        ctx.set_matvec_mode(MV_FP32_SIMT)


def test_subset_exact_f8_variants_bit_identical(exact_cohort):
    """The FP16 / E4M3 form on single CTAs and on CTA pairs gives the same products, bit for bit."""
    ctx, bed, _, cases = exact_cohort
    rng = np.random.default_rng(16)
    ctx.set_matvec_mode(MV_SUBSET_EXACT_F8)
    try:
        for k in (1, 40, 150):
            V = rng.standard_normal((N, k))
            outs = []
            for pair in (0, 1):
                ctx.set_tc_option(TC_SUBSET_PAIR, pair)
                outs.append(ctx.grm_matmul(V))
            np.testing.assert_array_equal(outs[1], outs[0])
    finally:
        ctx.set_tc_option(TC_SUBSET_PAIR, 2)
        ctx.set_matvec_mode(MV_FP32_SIMT)


def _bim_chrom():
    """22 chromosomes as contiguous blocks of the .bim markers."""
    return 1 + (np.arange(M) * 22) // M


def _subset_loco_range(g, b, e):
    """The subset's GRM markers inside .bim markers [b, e], as GRM-marker indices of its setgeno
    (updateChrStartEndIndexVec over the subset's own GRM markers)."""
    before = int(np.count_nonzero(g.qc_mask[:b]))
    return before, before + int(np.count_nonzero(g.qc_mask[b:e + 1])) - 1


def test_subset_exact_loco_products_match_oracle(exact_cohort):
    """A chromosome left out (.bim range) in the subset-exact engine: every phenotype's K_S,-j v
    against the oracle's LOCO GRM over setgeno of its subset (parallelCrossProd_LOCO); the range
    cleared, the products are the full K_S v again, bit for bit as before the range was set."""
    ctx, bed, _, cases = exact_cohort
    rng = np.random.default_rng(31)
    ranges = serve.loco_ranges(_bim_chrom())
    ctx.set_matvec_mode(MV_SUBSET_EXACT)
    try:
        ctx.engine_reserve(128, len(cases))
        Vs = []
        for _, mask, _ in cases:
            V = rng.standard_normal((N, 6)) + 0.4
            V[~mask] = 0.0
            Vs.append(V)

        def products():
            ids = []
            for slot, (_, mask, _) in enumerate(cases):
                ctx.engine_set_pheno(slot, np.ones(N), np.array([1.0, 0.5]), mask)
                ids.append(ctx.engine_submit(slot, 1, Vs[slot]))
            got = _run_products(ctx, np.concatenate(ids))
            return [np.column_stack([got[int(i)] for i in idk]) for idk in ids]

        full = products()
        for chrom in (4, 17):
            b, e = ranges[chrom]
            ctx.loco_set_bim(b, e)
            try:
                loco = products()
            finally:
                ctx.loco_clear()
            for (trait, mask, _), V, Y in zip(cases, Vs, loco):
                S = np.nonzero(mask)[0]
                g = plink.setgeno(bed, N, M, S + 1, mask, 0.01, 0.15)
                grm = aireml.DenseGRM(g)
                gb, ge = _subset_loco_range(g, b, e)
                ref = aireml.loco_grm(grm, g, gb, ge).K @ V[S]
                err = np.abs(Y[S] - ref).max() / np.abs(ref).max()
                print("LOCO chr %d %s: K_S,-j v max error %.2e" % (chrom, trait, err))
                assert err < 6e-5, (chrom, trait, err)
                # leaving the chromosome out changed the product
                assert np.abs(ref - grm.K @ V[S]).max() > 100 * err * np.abs(ref).max()
        again = products()
        for a, b_ in zip(full, again):
            np.testing.assert_array_equal(a, b_)
    finally:
        ctx.set_matvec_mode(MV_FP32_SIMT)


def test_subset_exact_loco_coefficients_match_oracle(exact_cohort, tmp_path):
    """Get_Coef_LOCO (FIT.R:40-73, run per chromosome by FIT.R:1208-1295) for phenotypes on their
    own subsets, through the subset-exact engine with a .bim range left out, against the oracle's
    Get_Coef_LOCO on the LOCO GRM of setgeno over each subset, both from the oracle's full fit."""
    ctx, bed, _, cases = exact_cohort
    ranges = serve.loco_ranges(_bim_chrom())
    sel = {c: ranges[c] for c in (2, 20)}
    use = cases[:2]  # a binary and a quantitative phenotype
    specs, fits, grms = [], [], []
    for trait, mask, f0 in use:
        S = np.nonzero(mask)[0]
        g = plink.setgeno(bed, N, M, S + 1, mask, 0.01, 0.15)
        grm = aireml.DenseGRM(g)
        grm.probe_index = S
        fit = (aireml.glmmkin_binary if trait == "binary" else aireml.glmmkin_quantitative)(grm, f0)
        specs.append(serve.FitSpec(f0, trait, mask=mask))
        fits.append(fit)
        grms.append((g, grm))
    ctx.set_matvec_mode(MV_SUBSET_EXACT)
    try:
        got = serve.fit_loco(ctx, specs, fits, sel, max_columns=256, bim=True)
    finally:
        ctx.set_matvec_mode(MV_FP32_SIMT)
    for c, (b, e) in sel.items():
        for k, ((trait, mask, f0), fit, (g, grm)) in enumerate(zip(use, fits, grms)):
            gb, ge = _subset_loco_range(g, b, e)
            ref = aireml.get_coef_loco(aireml.loco_grm(grm, g, gb, ge), f0, fit, trait)
            r = got[c][k]
            assert not isinstance(r, Exception), r
            rel = np.abs(r["coefficients"] - ref["alpha"]) / np.abs(ref["alpha"])
            print("LOCO chr %d %s: alpha rel error %s" % (c, trait, rel))
            np.testing.assert_allclose(r["coefficients"], ref["alpha"], rtol=1e-4)
            # both stop their solves on the same absolute residual rule (tol 1e-5), so entries of eta
            # near zero differ by about that much of eta's scale (measured 2.6e-6 at a scale of 0.35)
            np.testing.assert_allclose(r["linear_predictors"], ref["eta"], rtol=1e-4,
                                       atol=1e-5 * np.abs(ref["eta"]).max())
    # the step-1 model file with these LOCO results, as the reference saves it
    trait, mask, f0 = use[0]
    p = str(tmp_path / "loco.rda")
    output.write_model_rda(p, fits[0], f0, trait, ["s%d" % i for i in np.nonzero(mask)[0]],
                           loco={c: got[c][0] for c in sel})
    d = output.read_model_rda(p)
    assert len(d["LOCOResult"]) == 22 and d["LOCO"].all()
    for c in sel:
        e = d["LOCOResult"][c - 1]
        assert e["isLOCO"].all()
        np.testing.assert_array_equal(e["linear.predictors"].ravel(), got[c][0]["linear_predictors"])
        np.testing.assert_array_equal(e["alpha0"].ravel(), np.ravel(got[c][0]["coefficients"]))
    assert not d["LOCOResult"][0]["isLOCO"].any()


@pytest.mark.parametrize("trait", ["binary", "quantitative"])
def test_subset_exact_variance_ratio_matches_oracle(gpu_ctx, trait):
    """Variance ratio of a phenotype on its own subset (extractVarianceRatio after setgeno over the
    subset, FIT.R:2152-2423): the subset's variance-ratio markers and genotypes from the engine's
    subset QC, the solves on K_S, against the oracle over setgeno of the subset.  Runs last in this
    file: it sets the cohort up again with a variance-ratio marker draw."""
    ctx = gpu_ctx
    bed, _ = synth.synth_bed(78, N, M, 0.02)
    rng = np.random.default_rng(21)
    vr_rand = np.unique(rng.integers(0, M, 1000))
    mask = rng.uniform(size=N) > 0.25
    S = np.nonzero(mask)[0]
    ctx.set_matvec_mode(MV_FP32_SIMT)
    ctx.setgeno(bed, N, M, vr_random=vr_rand, min_mac_vr=20.0, is_var_ratio=True)
    g_all = plink.setgeno(bed, N, M, np.arange(1, N + 1), np.ones(N, bool), 0.01, 0.15)
    gv = synth.genetic_value_from_codes(g_all.codes, 5)
    y, C = synth.simulate_pheno(gv / gv.std(), 77, trait, tau=0.5, prevalence=0.25, h2=0.5)
    f0 = prep.make_fit0(y[S], C[S], trait, True)
    gs = plink.setgeno(bed, N, M, S + 1, mask, 0.01, 0.15, vr_rand, 20, True)
    grm = aireml.DenseGRM(gs)
    fit = (aireml.glmmkin_binary if trait == "binary" else aireml.glmmkin_quantitative)(grm, f0)
    order = np.random.default_rng(9).permutation(len(gs.vr_index))
    ref, rref = aireml.variance_ratio(grm, fit, trait, f0["Xorig"], gs.vr_codes, order)
    ctx.set_matvec_mode(MV_SUBSET_EXACT)
    try:
        ctx.engine_reserve(128, 1)
        ctx.engine_set_pheno(0, np.ones(N), np.array([1.0, 0.5]), mask)
        idx, mac = ctx.engine_subset_vr_markers(0)
        np.testing.assert_array_equal(idx, gs.vr_index)
        np.testing.assert_array_equal(ctx.engine_subset_geno(0, int(idx[3]))[S], gs.vr_codes[3])
        got, rgot = vr.variance_ratio_subset(ctx, 0, fit, trait, f0["Xorig"], mask, order)
    finally:
        ctx.set_matvec_mode(MV_FP32_SIMT)
    assert len(rgot) == len(rref)
    assert abs(got - ref) / ref < 1e-4, (got, ref)
