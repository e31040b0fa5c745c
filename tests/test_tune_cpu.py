"""Variant choice of the autotuner (host logic only)."""
from saigegpu import tune


def test_pick_keeps_first_variant_within_margin():
    v = tune.GRMV_VARIANTS
    # within timing noise of the first variant -> keep it
    assert tune._pick({v[0]: 30.0, v[1]: 29.7, v[2]: 29.6, v[3]: 29.5}, v) == v[0]
    # a clear win -> the fastest clear winner in order
    assert tune._pick({v[0]: 30.0, v[1]: 29.05, v[2]: 28.0, v[3]: 27.9}, v) == v[2]
    s = tune.SYRK_VARIANTS
    assert tune._pick({s[0]: 2.01, s[1]: 1.25, s[2]: 1.137, s[3]: 1.14}, s) == s[2]


def test_report_json_keys():
    rep = {"syrk": {"times_ms": {(0, 16): 1900.0, (1, 16): 1200.0}, "chosen": (1, 16)},
           "grmv": {32: {"times_ms": {(0, 128): 6.5, (1, 64): 6.4}, "chosen": (0, 128)}},
           "plan": [(32, 0, 128)]}
    out = tune.report_json(rep)
    assert out["syrk"]["chosen"] == {"pair": 1, "group": 16}
    assert out["grmv"]["32"]["times_ms"]["pair1_slice64"] == 6.4
    assert out["plan"] == [[32, 0, 128]]


def test_report_json_subset_table():
    rep = {"grmv": {}, "plan": [],
           "subset": {512: {"times_ms": {(0, 128): 49.7, (1, 128): 36.5}, "chosen": (1, 128)}},
           "subset_plan": [(512, 1, 128)]}
    out = tune.report_json(rep)
    assert out["subset"]["512"]["chosen"] == {"pair": 1, "slice": 128}
    assert out["subset_plan"] == [[512, 1, 128]]
