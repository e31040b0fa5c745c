"""Cluster-size choice of the autotuner (host logic only)."""
from saigegpu import tune


def test_pick_keeps_smaller_cluster_within_margin():
    # the split GRM.V at 128-256 columns: 2- and 4-CTA clusters within timing noise -> keep 2
    assert tune._pick({1: 30.0, 2: 29.05, 4: 29.06}, (1, 2, 4)) == 2
    assert tune._pick({1: 30.0, 2: 29.05, 4: 28.9}, (1, 2, 4)) == 2
    # the SYRK: 4-CTA clusters clearly faster -> 4
    assert tune._pick({1: 2.01, 2: 1.25, 4: 1.137}, (1, 2, 4)) == 4
    # nothing beats 1 by the margin -> 1
    assert tune._pick({1: 10.0, 2: 9.9, 4: 9.85}, (1, 2, 4)) == 1
