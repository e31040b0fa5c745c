"""The phenotype-file preamble of the null fit (prep.read_phenotypes) against the reference's own
example inputs and model, and its rules on small files (no GPU)."""
import os

import numpy as np

from saigegpu import prep

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_phenotype_preamble_reproduces_the_reference_model_inputs():
    """prep.read_phenotypes on the reference's example phenotype file and .fam, with the example
    commands' covariates (x1, x2 with x2 categorical), gives the reference model's samples in
    order, y, design column names and, through make_fit0, its design and covariate offset."""
    g = np.load(os.path.join(GOLDEN, "binary_fullGRM_model.npz"))
    d = prep.read_phenotypes(os.path.join(GOLDEN, "pheno_1000samples.txt"), os.path.join(GOLDEN, "samples_1000.fam"),
                             "y_binary", ["x1", "x2"], ["x2"])
    assert d["sample_ids"] == list(g["sample_ids"])
    np.testing.assert_array_equal(d["sub_1based"], np.arange(1, 1001))
    assert d["pheno_mask"].all()
    np.testing.assert_array_equal(d["y"], g["y"])
    assert ["minus1"] + d["covariate_names"] == list(g["X_names"])
    f0 = prep.make_fit0(d["y"], d["covariates"], "binary", True)
    np.testing.assert_allclose(f0["Xorig"], g["X"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(f0["offset"], g["offset"], rtol=0, atol=1e-12)


def test_phenotype_preamble_rules(tmp_path):
    """Complete cases only, the .fam's order, factor levels as R sorts and names them, the include
    list, one sex, the binary covariates' minimum count, inverse normalisation."""
    fam = tmp_path / "s.fam"
    fam.write_text("".join("f s%d 0 0 0 -9\n" % i for i in (4, 1, 3, 2, 0, 5)))
    rows = ["IID y q g sex c",
            "s0 1 0.5 b 1 1", "s1 0 1.5 a 1 0", "s2 1 NA a 0 1", "s3 0 2.5 c 0 1",
            "s4 1 3.5 a 1 0", "s5 0 4.5 b 1 1", "s9 1 5.5 a 1 1"]
    ph = tmp_path / "p.txt"
    ph.write_text("\n".join(rows) + "\n")
    d = prep.read_phenotypes(ph, fam, "y", ["q", "g"], ["g"])
    assert d["sample_ids"] == ["s4", "s1", "s3", "s0", "s5"]  # .fam order; s2 incomplete, s9 not genotyped
    np.testing.assert_array_equal(d["sub_1based"], [1, 2, 3, 5, 6])
    assert d["covariate_names"] == ["q", "gb", "gc"]
    np.testing.assert_array_equal(d["covariates"][:, 1], [0, 0, 0, 1, 1])
    np.testing.assert_array_equal(d["covariates"][:, 2], [0, 0, 1, 0, 0])
    d = prep.read_phenotypes(ph, fam, "y", ["q", "c"], ["c"], sample_include=["s0", "s1", "s4", "s5"],
                             sex_col="sex", female_only=True)
    assert d["sample_ids"] == ["s4", "s1", "s0", "s5"] and d["covariate_names"] == ["q", "c1"]
    # the binary covariate c has a cell (y = 0, c = 1) of one sample: dropped below two
    d = prep.read_phenotypes(ph, fam, "y", ["q", "c"], [], min_covariate_count=2)
    assert d["covariate_names"] == ["q"]
    d = prep.read_phenotypes(ph, fam, "q", [], [], trait="quantitative", inv_normalize=True)
    from scipy.stats import norm
    np.testing.assert_allclose(d["y"], norm.ppf((np.array([4, 2, 3, 1, 5]) - 0.5) / 5))
