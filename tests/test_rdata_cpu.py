"""The step-1 model file (.rda): R's serialisation read and written byte for byte, and the model laid
out as the reference's step 1 saves it (no GPU)."""
import gzip
import json
import os

import numpy as np
import pytest

from oracle import aireml, plink
from saigegpu import output, prep, rdata

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
RDA = os.path.join(GOLDEN, "example_binary_includenonAutoforvarRatio.rda")


def test_reference_model_file_round_trips_byte_for_byte():
    """The reference's own step-1 model file, read and written again, gives R's bytes exactly:
    the writer's flags, symbol references, string encodings, attributes and ALTREP items are R's."""
    raw = gzip.decompress(open(RDA, "rb").read())
    header, objs = rdata.read_rda(RDA)
    assert [k for k, _ in objs] == ["modglmm"]
    out = rdata.rda_bytes(objs, writer=header["writer"], min_reader=header["min_reader"],
                          encoding=header["encoding"])
    assert out == raw


def test_model_file_with_closures_round_trips_byte_for_byte():
    """An older step-1 model of the reference, holding the null glm object: closures, environments,
    a namespace, promises, calls and compiled byte code, all written back with R's bytes."""
    p = os.path.join(GOLDEN, "example_binary_includenonAutoforvarRatio_FemaleOnly.rda")
    raw = gzip.decompress(open(p, "rb").read())
    header, objs = rdata.read_rda(p)
    assert rdata.rda_bytes(objs, **header) == raw
    kinds = set()

    def walk(x, seen):
        if id(x) in seen:
            return
        seen.add(id(x))
        kinds.add(type(x).__name__ if not isinstance(x, rdata.RObj) else x.type)
        if isinstance(x, rdata.RObj):
            for e in (x.value if isinstance(x.value, list) else []):
                for part in (e if isinstance(e, tuple) else (e,)):
                    walk(part, seen)
            for _, v in x.attrs:
                walk(v, seen)
            walk(x.tail, seen)
        elif isinstance(x, rdata.REnv):
            for v in (x.enclos, x.frame, x.hashtab, x.attrib):
                walk(v, seen)

    seen = set()
    for _, o in objs:
        walk(o, seen)
    assert {rdata.CLOSXP, rdata.LANGSXP, rdata.PROMSXP, "REnv", "RNamedEnv", "RBytecode"} <= kinds


def test_format_2_round_trip():
    """save(..., version = 2) files: no native-encoding field in the header."""
    obj = rdata.r_named_list([("a", rdata.r_double([1.0, 2.0])), ("b", rdata.r_str(["x"]))])
    raw = rdata.rda_bytes([("m", obj)], version=2)
    assert raw[:5] == b"RDX2\n"
    header, objs = rdata.unserialize(raw[5:])
    assert header["version"] == 2 and "encoding" not in header
    assert rdata.rda_bytes(list(objs.value), **header) == raw


def test_values_round_trip(tmp_path):
    obj = rdata.r_named_list([
        ("d", rdata.r_double([1.5, -np.inf, np.nan], names=["a", "b", "c"])),
        ("i", rdata.r_int([1, rdata.NA_INTEGER, 7])),
        ("l", rdata.r_lgl([True, False])),
        ("s", rdata.r_str(["x", None, "été"])),
        ("m", rdata.r_matrix(np.arange(6.0).reshape(3, 2), ["u", "v"])),
        ("z", rdata.RObj(rdata.CPLXSXP, np.array([1 + 2j, -3j]))),
        ("r", rdata.RObj(rdata.RAWSXP, b"\x00\x01\xff")),
        ("nested", rdata.r_named_list([("names", rdata.r_str("again"))], cls=["k1", "k2"])),
        ("null", None),
    ])
    p = str(tmp_path / "x.rda")
    rdata.write_rda(p, [("obj", obj)])
    _, objs = rdata.read_rda(p)
    back = dict(objs)["obj"]
    assert back.names() == ["d", "i", "l", "s", "m", "z", "r", "nested", "null"]
    np.testing.assert_array_equal(back["d"].value, [1.5, -np.inf, np.nan])
    assert back["d"].names() == ["a", "b", "c"]
    assert list(back["i"].value) == [1, rdata.NA_INTEGER, 7]
    assert list(back["s"].value) == ["x", None, "été"]
    np.testing.assert_array_equal(rdata.to_numpy(back["m"]), np.arange(6.0).reshape(3, 2))
    np.testing.assert_array_equal(back["z"].value, [1 + 2j, -3j])
    assert back["r"].value == b"\x00\x01\xff"
    assert back["nested"].is_object and list(back["nested"].attr("class").value) == ["k1", "k2"]
    assert back["null"] is None
    # a symbol (SYMSXP, then its ASCII CHARSXP) is written once and referred to after: two matrices
    # carry "dim"
    two = rdata.r_list([rdata.r_matrix(np.eye(2)), rdata.r_matrix(np.eye(3))])
    raw = rdata.rda_bytes([("two", two)])
    assert raw.count(b"\x00\x00\x00\x01\x00\x04\x00\x09\x00\x00\x00\x03dim") == 1


def _strip_row_names(s):
    """Layout without what R's data frames add and this writer leaves out: row names (ALTREP row
    numbers) in names / dimnames, and model.matrix's "assign" attribute."""
    if not isinstance(s, dict):
        return s
    out = dict(s)
    out["attrs"] = [a for a in s["attrs"] if a != "assign"]
    if "dimnames" in s:
        out["dimnames"] = [None if d == "altrep" else _strip_row_names(d) for d in s["dimnames"]]
        if all(d is None for d in out["dimnames"]):  # only row names: no dimnames without them
            del out["dimnames"]
            out["attrs"] = [a for a in out["attrs"] if a != "dimnames"]
    if "fields" in s:
        out["fields"] = [[k, _strip_row_names(v)] for k, v in s["fields"]]
    return out


@pytest.fixture(scope="module")
def golden_fit(golden_plink):
    bed, n, m, ph = golden_plink
    g = plink.setgeno(bed, n, m, np.arange(1, n + 1), np.ones(n, bool), 0.01, 0.15)
    grm = aireml.DenseGRM(g)
    cov = np.column_stack([ph["x1"], ph["x2"]])
    return g, grm, cov, ph


def test_model_file_has_the_reference_layout_without_covariate_offset(golden_fit, tmp_path):
    """Binary trait, covariates in the design (isCovariateOffset = FALSE), no LOCO: the written
    model's fields, order, types, shapes, dimnames and classes are those of the reference's
    example_binary_includenonAutoforvarRatio.rda, except the fields that example's SAIGE version
    did not write yet (isCovariateOffset, offset, useSparseGRMtoFitNULL) and R's row names."""
    g, grm, cov, ph = golden_fit
    f0 = prep.make_fit0(ph["y_binary"], cov, "binary", False)
    fit = aireml.glmmkin_binary(grm, f0)
    ids = ["s%d" % i for i in range(grm.n)]
    p = str(tmp_path / "m.rda")
    output.write_model_rda(p, fit, f0, "binary", ids, covariate_names=["x1", "x2"])
    ours = rdata.schema(dict(rdata.read_rda(p)[1])["modglmm"])
    ref = rdata.schema(dict(rdata.read_rda(RDA)[1])["modglmm"])
    newer = {"isCovariateOffset", "offset", "useSparseGRMtoFitNULL"}
    ours_f = [[k, _strip_row_names(v)] for k, v in ours["fields"] if k not in newer]
    ref_f = [[k, _strip_row_names(v)] for k, v in ref["fields"]]
    ref_f = [[k, v] if k != "y" else [k, dict(v, attrs=[])] for k, v in ref_f]  # y's row names
    assert [k for k, _ in ours_f] == [k for k, _ in ref_f]
    for (k, a), (_, b) in zip(ours_f, ref_f):
        assert a == b, (k, a, b)
    # and the values read back
    d = output.read_model_rda(p)
    np.testing.assert_allclose(d["theta"], fit["theta"])
    back = output.covariate_transform_back(fit["coefficients"], f0["transform"], grm.n)
    np.testing.assert_allclose(d["coefficients"].ravel(), back)
    # the transform back recovers the untransformed design's coefficients: X_orig b = X_qr alpha
    Xo = np.column_stack([np.ones(grm.n), cov])
    np.testing.assert_allclose(Xo @ back, f0["X"] @ np.asarray(fit["coefficients"]).ravel(), rtol=1e-9, atol=1e-9)
    nk = d["obj.noK"]
    mu = np.asarray(fit["fitted_values"])
    np.testing.assert_allclose(nk["XVX"], f0["X"].T @ (f0["X"] * (mu * (1 - mu))[:, None]), rtol=1e-12)
    np.testing.assert_allclose(nk["XVX"] @ nk["XVX_inv"], np.eye(3), atol=1e-10)
    assert d["sampleID"] == ids and d["traitType"] == ["binary"]


def test_model_file_has_the_reference_layout_with_offset_and_loco(golden_fit, tmp_path):
    """Binary trait with the covariate offset and LOCO results (the reference's
    example_binary_fullGRM.rda): the same layout, each chromosome's LOCO entry included, plus the
    alpha0 the reference's current source adds to each entry (FIT.R:291)."""
    g, grm, cov, ph = golden_fit
    f0 = prep.make_fit0(ph["y_binary"], cov, "binary", True)
    fit = aireml.glmmkin_binary(grm, f0)
    # two chromosomes as two blocks of the GRM markers
    mq = g.codes.shape[0]
    loco = {}
    for c, (b, e) in {1: (0, mq // 2 - 1), 2: (mq // 2, mq - 1)}.items():
        r = aireml.get_coef_loco(aireml.loco_grm(grm, g, b, e), f0, fit, "binary")
        loco[c] = dict(isLOCO=True, coefficients=r["alpha"], linear_predictors=r["eta"], fitted_values=r["mu"],
                       Y=r["Y"], cov=r["cov"])
    p = str(tmp_path / "m.rda")
    output.write_model_rda(p, fit, f0, "binary", ["s%d" % i for i in range(grm.n)],
                           covariate_names=["x1", "x21"], loco=loco)
    ours = rdata.schema(dict(rdata.read_rda(p)[1])["modglmm"])
    ref = json.load(open(os.path.join(GOLDEN, "model_schema_binary_fullGRM.json")))
    ours_f = [[k, _strip_row_names(v)] for k, v in ours["fields"]]
    ref_f = [[k, _strip_row_names(v)] for k, v in ref["fields"]]
    ref_f = [[k, v] if k != "y" else [k, dict(v, attrs=[])] for k, v in ref_f]
    assert [k for k, _ in ours_f] == [k for k, _ in ref_f]
    for (k, a), (_, b) in zip(ours_f, ref_f):
        if k == "LOCOResult":
            assert a["len"] == b["len"] == 22
            ent_a, ent_b = a["fields"][0][1], b["fields"][0][1]
            assert ent_a["fields"][:-1] == ent_b["fields"], "LOCO entry"
            assert ent_a["fields"][-1][0] == "alpha0"
            assert a["fields"][2][1]["fields"][0][0] == "isLOCO"  # chromosomes without markers
            continue
        assert a == b, (k, a, b)
    d = output.read_model_rda(p)
    assert d["LOCO"].all() and d["isCovariateOffset"].all()
    np.testing.assert_allclose(d["LOCOResult"][0]["linear.predictors"].ravel(), loco[1]["linear_predictors"])
    assert not d["LOCOResult"][5]["isLOCO"].any()
    np.testing.assert_allclose(d["offset"].ravel(), f0["offset"])


def test_fit0_and_score_test_pieces_match_the_reference_model(golden_plink):
    """What the reference's example_binary_fullGRM.rda holds that does not depend on its GRM (the
    example commands fit it on a 22-chromosome genotype set whose .bed the checkout lacks) is
    reproduced exactly: y in sample order, the QR-transformed design Xorig (Covariate_Transform,
    FIT.R:1612-1648), the covariate offset of isCovariateOffset (FIT.R:1054-1065), and obj.noK from
    the model's own fitted values (ScoreTest_NULL_Model, FIT.R:579-591)."""
    _, _, _, ph = golden_plink
    g = np.load(os.path.join(GOLDEN, "binary_fullGRM_model.npz"))
    f0 = prep.make_fit0(ph["y_binary"], np.column_stack([ph["x1"], ph["x2"]]), "binary", True)
    np.testing.assert_array_equal(f0["y"], g["y"])
    np.testing.assert_allclose(f0["Xorig"], g["X"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(f0["offset"], g["offset"], rtol=0, atol=1e-12)
    mu = g["mu"]
    nk = output.score_test_null_model(mu, mu * (1 - mu), g["y"], g["X"])
    for k in ("XV", "XVX", "XXVX_inv", "XVX_inv", "S_a", "XVX_inv_XV", "V"):
        np.testing.assert_allclose(nk[k], g["noK_" + k], rtol=1e-9, atol=1e-12, err_msg=k)


def test_model_file_quantitative_without_covariates(tmp_path):
    """A quantitative trait with the intercept only (no QR transform, no offset) writes and reads back."""
    rng = np.random.default_rng(8)
    n = 60
    y = rng.standard_normal(n)
    f0 = prep.make_fit0(y, None, "quantitative", True)
    fit = dict(theta=np.array([0.7, 0.3]), coefficients=np.array([y.mean()]), linear_predictors=np.full(n, y.mean()),
               fitted_values=np.full(n, y.mean()), Y=y.copy(), residuals=y - y.mean(), cov=np.array([[0.01]]),
               converged=True)
    p = str(tmp_path / "q.rda")
    output.write_model_rda(p, fit, f0, "quantitative", ["s%d" % i for i in range(n)])
    d = output.read_model_rda(p)
    assert d["traitType"] == ["quantitative"] and not d["isCovariateOffset"].any()
    assert d["X"].shape == (n, 1) and d["coefficients"].shape == (1, 1)
    np.testing.assert_allclose(d["obj.noK"]["V"], np.full(n, 1 / 0.7))
    np.testing.assert_allclose(d["offset"].ravel(), 0.0)
    m = dict(rdata.read_rda(p)[1])["modglmm"]
    assert list(m["X"].attr("dimnames").value[1].value) == ["(Intercept)"]


def test_step1_outputs_under_a_prefix(tmp_path):
    """<prefix>.rda and <prefix>.varianceRatio.txt, as the reference's outputPrefix names them."""
    rng = np.random.default_rng(3)
    n = 40
    y = (rng.uniform(size=n) < 0.4).astype(float)
    f0 = prep.make_fit0(y, rng.standard_normal((n, 1)), "binary", True)
    mu = np.full(n, y.mean())
    fit = dict(theta=np.array([1.0, 0.2]), coefficients=np.array([0.1]), linear_predictors=np.zeros(n),
               fitted_values=mu, Y=y - mu, residuals=y - mu, cov=np.array([[0.02]]), converged=True)
    paths = output.write_step1(tmp_path / "run", fit, f0, "binary", ["s%d" % i for i in range(n)],
                               variance_ratios=[0.95, 0.97])
    assert [os.path.basename(p) for p in paths] == ["run.rda", "run.varianceRatio.txt"]
    assert output.read_variance_ratio(paths[1]) == [0.95, 0.97]
    assert output.read_model_rda(paths[0])["traitType"] == ["binary"]
