"""bench.py's host-side arithmetic, on CPU: the paths a road needs for a 1%
Monte Carlo error (the reference's per-road N*, from a pilot's standard
error) and the roofline record the bench prints for its issue-bound kernels.
"""
import json
import math

import numpy as np

import bench


def test_n_star_from_the_pilot_standard_error():
    P = bench.PILOT_PATHS
    res = np.zeros((3, 2, 5))
    # road 0: species 1 needs (1.5 sqrt(P) / 1)^2 = 2.25 P paths
    res[0, 0, 2], res[0, 0, 4] = 100.0, 0.5
    res[0, 1, 2], res[0, 1, 4] = 100.0, 1.5
    # road 1: tiny error -> the floor
    res[1, :, 2], res[1, :, 4] = 50.0, 1e-6
    # road 2: extinct everywhere (mean 0) -> the floor
    need = bench.n_star(res, floor=64)
    assert 2.25 * P <= need[0] <= 2.25 * P + 1
    assert need[1] == 64 and need[2] == 64


def test_rov_n_star_ignores_zero_and_non_finite_values():
    res = np.zeros((4, 1, 14))
    res[0, 0, 10], res[0, 0, 13] = 200.0, 4.0          # (4 sqrt(500) / 2)^2 = 2000
    res[1, 0, 10], res[1, 0, 13] = 0.0, 1.0
    res[2, 0, 10], res[2, 0, 13] = float("nan"), 1.0
    res[3, 0, 10], res[3, 0, 13] = -200.0, 0.01
    need = bench.rov_n_star(res, pilot=500, floor=128)
    assert 2000 <= need[0] <= 2001
    assert need[1:] == [128, 128, 128]


def test_roofline_line_is_issue_bound_and_serialisable():
    units = {"rov_forward_sparse": 921_600, "knn": 24_745_196}
    split = {"rov_forward_sparse": (50.0, 1), "knn": (42.0, 48), "mte_sparse": (2.8, 1)}
    top = ("rov_forward_sparse", split["rov_forward_sparse"])
    out = bench.roofline_line(top, split, units, 2070.0, 1e12, 2e10, 1900.0, 6800.0,
                              "measured")
    peak = bench.SMS * bench.SCHEDULERS * 2070.0 / 1e3
    assert math.isclose(out["peak"], peak)
    fw = bench.ROOF["rov_forward_sparse"]
    ach = fw["inst_per_unit"] * units["rov_forward_sparse"] / 0.050 / 1e9
    assert math.isclose(out["achieved"], ach) and math.isclose(out["frac"], ach / peak)
    assert out["kernel"] == "k_rov_forward_union" and out["bound"] == "issue"
    assert math.isclose(out["traffic"], fw["bytes_per_unit"] * units["rov_forward_sparse"])
    (knn,) = out["others"]
    assert knn["kernel"] == "k_knn_rov" and knn["launches_per_step"] == 48
    kr = bench.ROOF["knn"]
    assert math.isclose(knn["traffic"], kr["bytes_per_unit"] * units["knn"] / 48)
    assert 0.0 < knn["frac"] < 1.0 and 0.0 < out["frac"] < 1.0
    assert math.isclose(out["mte_sparse"]["dense_equiv_tflops"], 1e12 / 2.8e-3 / 1e12)
    json.dumps(out)


def test_roofline_line_without_a_count_has_no_fraction():
    split = {"other": (3.0, 2)}
    out = bench.roofline_line(("other", split["other"]), split, {}, 2070.0, 0.0, 0.0,
                              1900.0, 6800.0, "fallback")
    assert out["achieved"] is None and out["frac"] is None and out["traffic"] is None
    assert out["mte_sparse"]["dense_equiv_tflops"] is None
    json.dumps(out)
