"""CPU tests of the oracle: pinned against the reference's own fixtures and against direct algebra."""
import json
import os

import numpy as np
import pytest

from oracle import aireml, plink, probes
from saigegpu import prep, synth

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_decode_matches_plink_frq(golden_plink):
    """Known-answer test: A1 MAF of the reference's example .bed equals PLINK's .frq (all 10k markers)."""
    bed, n, m, _ = golden_plink
    codes = plink.decode_bed(bed, n, m)
    ok = codes != 3
    p = np.where(ok, codes, 0).sum(1) / (2.0 * ok.sum(1))
    frq = np.load(os.path.join(GOLDEN, "plink_1000x10k_frq.npy"))
    assert np.array_equal(np.round(np.minimum(p, 1 - p), 4), frq)


def test_setgeno_qc_and_imputation():
    bed, codes = synth.synth_bed(7, 37, 60, 0.05)
    sub = np.arange(1, 38)[::-1].copy()
    g = plink.setgeno(bed, 37, 60, sub, np.ones(37, bool), 0.05, 0.15)
    assert g.codes.shape[1] == 37
    kept = np.nonzero(g.qc_mask)[0]
    for row, j in enumerate(kept):
        c = codes[j][sub - 1]
        miss = c == 3
        np.testing.assert_array_equal(g.codes[row][~miss], c[~miss])
        nm = c[~miss].astype(float)
        fill = int(np.floor(np.float64(np.float32(2) * np.float32(nm.sum()) / np.float32(2 * len(nm))) + 0.5))
        assert np.all(g.codes[row][miss] == fill)
    assert (g.freq >= 0).all() and (g.freq <= 1).all()


def test_vr_markers_leave_the_grm():
    bed, codes = synth.synth_bed(9, 200, 80, 0.0)
    allm = plink.setgeno(bed, 200, 80, np.arange(1, 201), np.ones(200, bool), 0.01, 0.15)
    vr = np.array([1, 5, 9, 33, 70])
    g = plink.setgeno(bed, 200, 80, np.arange(1, 201), np.ones(200, bool), 0.01, 0.15, vr, 20, True)
    for j in vr:
        if allm.qc_mask[j] and g.vr_index.size and j in g.vr_index:
            assert not g.qc_mask[j]
    assert g.codes.shape[0] + len(g.vr_index) >= allm.codes.shape[0]


def test_pack_roundtrip():
    rng = np.random.default_rng(0)
    codes = rng.integers(0, 3, size=(5, 13)).astype(np.uint8)
    packed = plink.pack_codes(codes)
    fields = np.stack([(packed >> (2 * j)) & 3 for j in range(4)], axis=2).reshape(5, -1)[:, :13]
    back = 2 - ((fields & 1) + (fields >> 1))
    np.testing.assert_array_equal(back, codes)


def _small_problem(seed=3, n=150, m=400):
    bed, _ = synth.synth_bed(seed, n, m, 0.01)
    g = plink.setgeno(bed, n, m, np.arange(1, n + 1), np.ones(n, bool), 0.01, 0.15)
    return aireml.DenseGRM(g), g


def test_oracle_pcg_solves_sigma():
    grm, _ = _small_problem()
    n = grm.n
    rng = np.random.default_rng(1)
    w = rng.uniform(0.1, 0.3, n)
    tau = np.array([1.0, 0.4])
    b = rng.standard_normal((n, 3))
    x, it = aireml.pcg(grm, w, tau, b, 500, 1e-20, return_iters=True)
    S = np.diag(tau[0] / w) + tau[1] * grm.K
    np.testing.assert_allclose(x, np.linalg.solve(S, b), rtol=1e-8, atol=1e-10)
    for j in range(3):
        xj, itj = aireml.pcg(grm, w, tau, b[:, j], 500, 1e-20, return_iters=True)
        assert itj == it[j]
        np.testing.assert_allclose(xj, x[:, j], rtol=1e-12)


def test_oracle_hutchinson_trace_is_unbiased():
    grm, _ = _small_problem()
    n = grm.n
    w = np.full(n, 0.2)
    tau = np.array([1.0, 0.3])
    X = np.ones((n, 1))
    S = np.diag(tau[0] / w) + tau[1] * grm.K
    Si = np.linalg.inv(S)
    SX = Si @ X
    cov = np.linalg.inv(X.T @ SX)
    P = Si - SX @ cov @ SX.T
    exact = np.trace(P @ grm.K)
    est, nr = aireml.get_trace(grm, SX, X, w, tau, cov, 30, 500, 1e-12, 0.0025)
    assert nr >= 30
    assert abs(est - exact) / exact < 0.05


def test_probes_are_rademacher_and_deterministic():
    u = probes.rademacher(200, 3, 1000)
    assert set(np.unique(u)) == {-1.0, 1.0}
    np.testing.assert_array_equal(u, probes.rademacher(200, 3, 1000))
    assert abs(u.mean()) < 0.1
    assert not np.array_equal(u, probes.rademacher(200, 4, 1000))
    assert np.array_equal(probes.hash3(1, 2, np.arange(5)), synth.hash3(1, 2, np.arange(5)))


def test_glm_score_equations():
    rng = np.random.default_rng(2)
    n = 500
    C = rng.standard_normal((n, 2))
    y = (rng.uniform(size=n) < 1 / (1 + np.exp(-(-1 + C @ [0.5, -0.3])))).astype(float)
    f0 = prep.make_fit0(y, C, "binary", covariate_offset=False)
    mu = 1 / (1 + np.exp(-f0["linear_predictors"]))
    np.testing.assert_allclose(f0["X"].T @ (y - mu), 0, atol=1e-6)


def test_golden_theta_monte_carlo_band(golden_plink):
    """The reference's example fits pin tau only loosely (probes and VR markers come from R's RNG).

    Over 20 probe seeds and random VR-marker draws (none, single-ratio and categorical exclusion
    from the GRM) the oracle gives binary tau1 0.258 +- 0.040 (golden 0.335: +1.9 sd) and
    quantitative tau (0.238 +- 0.006, 0.451 +- 0.009) against the golden (0.201, 0.483), whose sum
    agrees to 0.6%.  The golden fits were made on another genotype set of the same samples (the
    example commands' 22-chromosome nfam_100 set, 128,868 markers, whose .bed the checkout lacks),
    not on this 10k-marker set, so their GRM differs; the quantitative band below is that gap."""
    bed, n, m, ph = golden_plink
    gold = json.load(open(os.path.join(GOLDEN, "golden_fits.json")))
    g = plink.setgeno(bed, n, m, np.arange(1, n + 1), np.ones(n, bool), 0.01, 0.15)
    grm = aireml.DenseGRM(g)
    cov = np.column_stack([ph["x1"], ph["x2"]])
    fb = prep.make_fit0(ph["y_binary"], cov, "binary", True)
    rb = aireml.glmmkin_binary(grm, fb)
    t_gold = gold["example_binary_fullGRM"]["theta"][1]
    # Monte-Carlo spread of tau1 over probe seeds and VR draws here is 0.040 (sd); allow 3 sd
    assert abs(rb["theta"][1] - t_gold) < 3 * 0.040
    assert abs(rb["coefficients"][0] - gold["example_binary_fullGRM"]["coefficients"][0]) < 0.05
    fq = prep.make_fit0(ph["y_quantitative"], cov, "quantitative", True)
    rq = aireml.glmmkin_quantitative(grm, fq)
    tq = np.array(gold["example_quantitative_fullGRM"]["theta"])
    rel = np.abs(rq["theta"] - tq) / tq
    assert rel[0] < 0.25 and rel[1] < 0.10, rel
    assert abs(rq["theta"].sum() - tq.sum()) / tq.sum() < 0.02


def test_c_restatement_of_reference_cpu_path():
    from oracle import cpu_ref
    grm, g = _small_problem(5, 120, 300)
    cg = cpu_ref.CpuGeno(g)
    rng = np.random.default_rng(3)
    b = rng.standard_normal(grm.n)
    np.testing.assert_allclose(cg.crossprod(b), grm.K @ b, rtol=1e-4, atol=1e-4 * np.abs(grm.K @ b).max())
    w = rng.uniform(0.1, 0.3, grm.n)
    tau = np.array([1.0, 0.3])
    x, it = cg.pcg(w, tau, b, 500, 1e-5)
    xo, ito = aireml.pcg(grm, w, tau, b, 500, 1e-5, return_iters=True)
    assert abs(it - ito) <= 2
    assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < 1e-3


def test_c_synth_setgeno_matches_python_recipe():
    from oracle import cpu_ref
    n, m = 203, 150
    pg = cpu_ref.PackedGeno.synthetic(77, n, m, 0.03)
    bed, _ = synth.synth_bed(77, n, m, 0.03)
    g = plink.setgeno(bed, n, m, np.arange(1, n + 1), np.ones(n, bool), 0.01, 0.15)
    assert pg.m == g.codes.shape[0]
    np.testing.assert_array_equal(pg.packed, plink.pack_codes(g.codes))
    np.testing.assert_array_equal(pg.lut[:, :3], plink.std_lut(g.freq, g.invstd))


def test_variance_ratio_oracle_on_golden(golden_plink):
    """VR of the reference's example (binary, covariates as offsets) lands near the golden null VR."""
    bed, n, m, ph = golden_plink
    rng = np.random.default_rng(5)
    vr_rand = np.unique(rng.integers(0, m, 1000))
    g = plink.setgeno(bed, n, m, np.arange(1, n + 1), np.ones(n, bool), 0.01, 0.15, vr_rand, 20, True)
    grm = aireml.DenseGRM(g)
    cov = np.column_stack([ph["x1"], ph["x2"]])
    f0 = prep.make_fit0(ph["y_binary"], cov, "binary", True)
    fit = aireml.glmmkin_binary(grm, f0)
    order = rng.permutation(len(g.vr_index))
    vr, ratios = aireml.variance_ratio(grm, fit, "binary", f0["Xorig"], g.vr_codes, order)
    assert len(ratios) >= 30
    gold = json.load(open(os.path.join(GOLDEN, "golden_fits.json")))["variance_ratio_null"]
    # golden runs differ in tau by up to 30% (R's RNG for probes and markers): loose band
    assert 0.85 < vr < 1.05, vr
    assert abs(vr - gold["example_binary"][0]) < 0.1


def test_output_writers_roundtrip(tmp_path):
    from saigegpu import output
    p = tmp_path / "x.varianceRatio.txt"
    output.write_variance_ratio(p, [0.9456, 1.01])
    assert output.read_variance_ratio(p) == [0.9456, 1.01]
    fit = dict(theta=[1, 0.3], coefficients=[-2.5], linear_predictors=[0.1, 0.2], fitted_values=[0.5, 0.6],
               Y=[1, 2], residuals=[0.1, 0.1], cov=[[0.01]], converged=True)
    output.write_model(tmp_path / "m.json", fit, "binary", ["a", "b"])
    d = output.read_model(tmp_path / "m.json")
    assert d["theta"].tolist() == [1, 0.3] and d["sampleID"] == ["a", "b"]


def test_categorical_variance_ratio_oracle_on_golden(golden_plink):
    """Two MAC categories (10 < MAC <= 20.5 and MAC > 20.5, the fitNULLGLMM defaults) on the
    reference's example: every marker of the first category and the random draw's markers above
    leave the GRM; each category's null VR lands near the golden two-category file
    (example_binary_fullGRM.varianceRatio.txt: 0.9456 and 0.9400)."""
    from saigegpu import vr as vrmod
    bed, n, m, ph = golden_plink
    rng = np.random.default_rng(5)
    vr_rand = np.unique(rng.integers(0, m, 1000))
    g = plink.setgeno(bed, n, m, np.arange(1, n + 1), np.ones(n, bool), 0.01, 0.15, vr_rand, 10.0, True,
                      max_mac_vr=20.5)
    cats = vrmod.category_markers(g.vr_mac)
    assert len(cats) == 2 and all(len(c) >= 30 for c in cats)
    assert np.all(g.vr_mac[cats[0]] <= 20) and np.all(g.vr_mac[cats[1]] > 20)
    # categorical selection: every marker with 10 <= MAC < 20.5 is a variance-ratio marker
    g1 = plink.setgeno(bed, n, m, np.arange(1, n + 1), np.ones(n, bool), 0.01, 0.15, None, 10.0, True,
                       max_mac_vr=20.5)
    assert np.all((g1.vr_mac >= 10) & (g1.vr_mac < 20.5))
    grm = aireml.DenseGRM(g)
    cov = np.column_stack([ph["x1"], ph["x2"]])
    f0 = prep.make_fit0(ph["y_binary"], cov, "binary", True)
    fit = aireml.glmmkin_binary(grm, f0)
    orders = [c[rng.permutation(len(c))] for c in cats]
    vrs = aireml.categorical_variance_ratio(grm, fit, "binary", f0["Xorig"], g.vr_codes, orders)
    gold = json.load(open(os.path.join(GOLDEN, "golden_fits.json")))["variance_ratio_null"]["example_binary_fullGRM"]
    # measured 0.952-0.962 over three random draws against the golden 0.9456 / 0.9400: the
    # golden run's probes, marker draw and tau (0.335 there, 0.24-0.29 here) come from R's RNG
    for v, gv in zip(vrs, gold):
        assert abs(v - gv) < 0.03, (vrs, gold)


def test_loco_on_a_subset_equals_its_grm_without_the_chromosome():
    """What the subset-exact engine's LOCO relies on, in the oracle: the reference's LOCO GRM of a
    phenotype's setgeno ((M K - Z_j' Z_j) / (M - M_j), diag minus the chromosome's sum z^2;
    parallelCrossProd_LOCO FIT.cpp:1790-1851, getDiagOfSigma_LOCO FIT.cpp:2370-2392) equals the GRM
    of that setgeno built over its GRM markers outside the chromosome."""
    n, m = 160, 900
    bed, _ = synth.synth_bed(21, n, m, 0.03)
    mask = np.random.default_rng(4).uniform(size=n) > 0.3
    S = np.nonzero(mask)[0]
    g = plink.setgeno(bed, n, m, S + 1, mask, 0.01, 0.15)
    grm = aireml.DenseGRM(g)
    b_bim, e_bim = 300, 520  # one chromosome as .bim markers
    gb = int(np.count_nonzero(g.qc_mask[:b_bim]))
    ge = gb + int(np.count_nonzero(g.qc_mask[b_bim:e_bim + 1])) - 1
    loco = aireml.loco_grm(grm, g, gb, ge)
    z = plink.std_geno(g).astype(np.float64)
    keep = np.ones(z.shape[0], bool)
    keep[gb:ge + 1] = False
    zk = z[keep]
    np.testing.assert_allclose(loco.K, zk.T @ zk / zk.shape[0], rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(loco.diag_sum, (zk * zk).sum(axis=0), rtol=1e-10)
    assert loco.m_qc == zk.shape[0]


def test_refinement_study_runs():
    """The refinement study (host emulation of one-product inner solves) runs and both solves reach
    the direct solve's accuracy class on a small problem."""
    from saigegpu import refinement_study
    res = refinement_study.study(n=200, m=500, trials=2)
    assert [r["trait"] for r in res] == ["binary", "quantitative"]
    for r in res:
        for s in r["solves"]:
            assert s["err_direct"] < 1e-3 and s["err_refined"] < 1e-3
    # BF16 keeps 8 significant bits: 1 + 2^-9 rounds down, 1 + 3 2^-9 up to 1 + 2^-7, and the tie
    # 1 + 2^-8 to the even neighbour 1
    b = refinement_study.bf16(np.array([1.0 + 2 ** -9, 1.0 + 3 * 2 ** -9, 1.0 + 2 ** -8]))
    np.testing.assert_array_equal(b, [1.0, 1.0 + 2 ** -7, 1.0])
