"""The oracle reproduces the committed golden fixtures (CPU only)."""
import os

import numpy as np

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(G, f"{name}.npz"))


def test_reduce_golden(orc):
    g = load("reduce")
    assert abs(orc.reduce_sum(g["x64"]) - g["sum64"]) <= 4096 * 2 ** -53 * g["abs64"]
    hi, lo = orc.exact_sum(g["x64"])
    assert hi == g["sum64"]
    assert orc.exact_dot(g["x64"], g["y64"])[0] == g["dot64"]
    assert orc.exact_dot(g["x32"], g["y32"])[0] == g["dot32"]
    assert orc.reduce_minloc(g["x64"]) == (g["min64"], g["argmin64"])
    assert orc.reduce_maxloc(g["x64"]) == (g["max64"], g["argmax64"])
    assert orc.reduce_minloc(g["t32"]) == (g["min_t32"], g["argmin_t32"])
    assert orc.reduce_maxloc(g["t32"]) == (g["max_t32"], g["argmax_t32"])
    assert orc.reduce_sum(g["i32"]) == g["sum_i32"]
    assert orc.reduce_bitor(g["i32"]) == g["or_i32"]
    assert orc.reduce_bitand(g["i32"]) == g["and_i32"]


def test_scan_golden(orc):
    g = load("scan")
    np.testing.assert_array_equal(orc.scan(g["a"], "plus"), g["a_incl"])
    np.testing.assert_array_equal(orc.scan(g["a"], "plus", exclusive=True, init=0), g["a_excl"])
    np.testing.assert_array_equal(orc.scan(g["b"], "plus", exclusive=True, init=7), g["b_excl7"])
    np.testing.assert_array_equal(orc.scan(g["iota"], "min"), g["iota_min"])
    np.testing.assert_array_equal(orc.scan(g["iota"], "max"), g["iota_max"])
    np.testing.assert_array_equal(orc.scan(g["rev"], "min"), g["rev_min"])


def test_sort_golden(orc):
    g = load("sort")
    k, v = orc.sort_pairs(g["ku"], np.arange(g["ku"].size, dtype=np.int32))
    np.testing.assert_array_equal(k, g["ku_sorted"])
    np.testing.assert_array_equal(v, g["ku_perm"])
    k, v = orc.sort_pairs(g["kf"], np.arange(g["kf"].size, dtype=np.int32))
    np.testing.assert_array_equal(k, g["kf_sorted"])
    np.testing.assert_array_equal(v, g["kf_perm"])
    np.testing.assert_array_equal(orc.sort(g["k64"]), g["k64_sorted"])
    np.testing.assert_array_equal(orc.sort(g["k64"], descending=True), g["k64_desc"])
    k, v = orc.sort_pairs(g["kd"], np.arange(g["kd"].size, dtype=np.int32))
    np.testing.assert_array_equal(k, g["kd_sorted"])
    np.testing.assert_array_equal(v, g["kd_perm"])
    k, v = orc.sort_pairs(g["kd"], np.arange(g["kd"].size, dtype=np.int32), descending=True)
    np.testing.assert_array_equal(k, g["kd_desc"])
    np.testing.assert_array_equal(v, g["kd_desc_perm"])


def test_histogram_golden(orc):
    g = load("histogram")
    np.testing.assert_array_equal(orc.histogram(g["z256"], 256).astype(np.int64), g["h256"])
    np.testing.assert_array_equal(orc.histogram(g["z64k"], 65536).astype(np.int64), g["h64k"])


def test_axpy_golden(orc):
    g = load("axpy")
    y = g["y"].copy()
    orc.axpy(float(g["a"]), g["x"], y)
    np.testing.assert_array_equal(y, g["y_out"])
