"""Reducers through the C ABI vs the oracle (seq_exec semantics) and the
golden fixtures.  Integer results, Min/Max values and MinLoc/MaxLoc indices
are bit-exact; floating-point sums are within the stated bounds of the exact
sum."""
import math
import os

import numpy as np
import pytest

from conftest import to_dev

pytestmark = pytest.mark.gpu

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
U32 = 2.0 ** -24
U64 = 2.0 ** -53
SIZES = [0, 1, 31, 32, 33, 255, 256, 257, 4095, 4096, 4097, 65537, (1 << 20) + 1]


def data(dt, n, seed):
    rng = np.random.default_rng(seed)
    if np.dtype(dt).kind == "f":
        return rng.uniform(-1, 1, n).astype(dt)
    if np.dtype(dt).kind == "u":
        return rng.integers(0, np.iinfo(dt).max, n, dtype=np.uint64).astype(dt)
    return rng.integers(np.iinfo(dt).min, np.iinfo(dt).max, n, dtype=np.int64).astype(dt)


def naive_bound(n, u, abs_sum):
    # any summation order: |err| <= (n-1) u sum|x| (Higham 4.3)
    return max(n - 1, 1) * u * abs_sum


def test_golden_reduce(prims):
    g = np.load(os.path.join(G, "reduce.npz"))
    x64, x32 = to_dev(g["x64"]), to_dev(g["x32"])
    n = g["x64"].size
    for mode in (0, 1, 2, 3):
        assert abs(prims.reduce_sum(x64, mode=mode) - g["sum64"]) <= naive_bound(n, U64, g["abs64"])
        assert abs(prims.reduce_sum(x32, mode=mode) - g["sum32"]) <= naive_bound(n, U32, g["abs32"])
    # compensated FP32 is within a few ulps of the exact sum here
    assert abs(prims.reduce_sum(x32, mode=1) - g["sum32"]) <= 1e-12 * g["abs32"]
    assert abs(prims.dot(x64, to_dev(g["y64"]), mode=1) - g["dot64"]) <= 1e-14 * g["abs64"]
    assert prims.reduce_minloc(x64) == (g["min64"], g["argmin64"])
    assert prims.reduce_maxloc(x64) == (g["max64"], g["argmax64"])
    t32 = to_dev(g["t32"])
    assert prims.reduce_minloc(t32) == (g["min_t32"], g["argmin_t32"])
    assert prims.reduce_maxloc(t32) == (g["max_t32"], g["argmax_t32"])
    i32 = to_dev(g["i32"])
    assert prims.reduce_sum(i32) == g["sum_i32"]
    assert prims.reduce_bitor(i32) == g["or_i32"]
    assert prims.reduce_bitand(i32) == g["and_i32"]


@pytest.mark.parametrize("dt", [np.int32, np.int64, np.uint32, np.uint64])
def test_integer_reducers_bit_exact(prims, orc, dt):
    for i, n in enumerate(SIZES):
        x = data(dt, n, i)
        d = to_dev(x)
        assert prims.reduce_sum(d) == orc.reduce_sum(x), n
        assert prims.reduce_min(d) == orc.reduce_min(x), n
        assert prims.reduce_max(d) == orc.reduce_max(x), n
        assert prims.reduce_bitor(d) == orc.reduce_bitor(x), n
        assert prims.reduce_bitand(d) == orc.reduce_bitand(x), n
        if np.dtype(dt).kind == "i":
            assert prims.reduce_minloc(d) == orc.reduce_minloc(x), n
            assert prims.reduce_maxloc(d) == orc.reduce_maxloc(x), n


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_float_minmax_loc_bit_exact_with_ties(prims, orc, dt):
    for i, n in enumerate(SIZES):
        rng = np.random.default_rng(100 + i)
        # few distinct values: ties everywhere, lowest index must win
        x = rng.integers(-3, 4, n).astype(dt)
        d = to_dev(x)
        assert prims.reduce_minloc(d) == orc.reduce_minloc(x), n
        assert prims.reduce_maxloc(d) == orc.reduce_maxloc(x), n
        y = data(dt, n, 200 + i)
        dy = to_dev(y)
        assert prims.reduce_minloc(dy) == orc.reduce_minloc(y), n
        assert prims.reduce_maxloc(dy) == orc.reduce_maxloc(y), n
        assert prims.reduce_min(dy) == orc.reduce_min(y)
        assert prims.reduce_max(dy) == orc.reduce_max(y)


def test_signed_zero_first_wins(prims, orc):
    import torch
    for vals in ([0.0, -0.0, 1.0], [-0.0, 0.0, 1.0]):
        for dt in (np.float32, np.float64):
            x = np.array(vals * 5000, dtype=dt)
            got = prims.reduce_min(to_dev(x))
            assert math.copysign(1.0, got) == math.copysign(1.0, orc.reduce_min(x))
            assert prims.reduce_minloc(to_dev(x)) == orc.reduce_minloc(x)


def test_empty_identity(prims):
    import torch
    e = torch.zeros(0, dtype=torch.float32, device="cuda")
    assert prims.reduce_minloc(e) == (float(np.finfo(np.float32).max), -1)
    assert prims.reduce_maxloc(e) == (float(-np.finfo(np.float32).max), -1)
    assert prims.reduce_sum(e) == 0.0


@pytest.mark.parametrize("dt,u", [(np.float32, U32), (np.float64, U64)])
def test_float_sums_vs_exact(prims, orc, dt, u):
    for i, n in enumerate(SIZES):
        x = data(dt, n, 300 + i)
        y = data(dt, n, 400 + i)
        hi, lo = orc.exact_sum(x)
        a = float(np.abs(x.astype(np.float64)).sum())
        d, dy = to_dev(x), to_dev(y)
        assert abs(prims.reduce_sum(d) - hi) <= naive_bound(n, u, a) + 1e-300
        # compensated: per-thread TwoSum error O(m u^2) plus the FP64 combine
        assert abs(prims.reduce_sum(d, mode=1) - hi) <= (n * u * u + 64 * U64) * a + 1e-300
        dh, _ = orc.exact_dot(x, y)
        ad = float(np.abs(x.astype(np.float64) * y.astype(np.float64)).sum())
        assert abs(prims.dot(d, dy) - dh) <= naive_bound(n, u, ad) + 1e-300
        assert abs(prims.dot(d, dy, mode=1) - dh) <= (n * u * u + 64 * U64) * ad + 1e-300


def test_deterministic_mode_independent_of_alignment(prims):
    import torch
    rng = np.random.default_rng(7)
    for dt in (np.float32, np.float64):
        x = rng.uniform(-1, 1, (1 << 20) + 5).astype(dt)
        big = to_dev(np.concatenate([np.zeros(3, dt), x]))
        aligned = to_dev(x)
        for mode in (2, 3):
            r1 = prims.reduce_sum(aligned, mode=mode)
            r2 = prims.reduce_sum(big[3:], mode=mode)  # 3 elements off 16-byte alignment
            r3 = prims.reduce_sum(aligned, mode=mode)
            assert r1 == r2 == r3


def test_misaligned_and_offset_views(prims, orc):
    rng = np.random.default_rng(8)
    x = rng.uniform(-1, 1, 100003)
    d = to_dev(x)
    for off in (1, 2, 3):
        v, l = prims.reduce_minloc(d[off:])
        assert (v, l) == orc.reduce_minloc(x[off:])
        assert abs(prims.reduce_sum(d[off:]) - math.fsum(x[off:].tolist())) < 1e-10
        assert abs(prims.dot(d[off:], d[:-off]) - math.fsum((x[off:] * x[:-off]).tolist())) < 1e-10


def test_device_output_no_sync(prims):
    import torch
    x = torch.rand(1 << 16, device="cuda", dtype=torch.float64)
    out = torch.empty(1, dtype=torch.float64, device="cuda")
    prims.reduce_sum(x, out=out)
    torch.cuda.synchronize()
    assert abs(out.item() - x.sum().item()) < 1e-9


def test_compensated_f32_beats_naive_f64_ill_conditioned(prims, orc):
    """FP32 sum with condition number ~1e10 (the last element cancels the
    rest): the compensated FP32 sum (cascaded TwoSum per thread,
    double-double across threads) is at least as accurate as the naive FP64
    sum of the same values and within 1e-6 relative of the exact sum."""
    rng = np.random.default_rng(21)
    n = 1 << 22
    sign = rng.choice([-1.0, 1.0], n)
    x = (sign * np.clip(np.exp(rng.normal(0, 6, n)), 1e-8, 1e8)).astype(np.float32)
    head, _ = orc.exact_sum(x[:-1])
    x[-1] = np.float32(-head)
    ex, exlo = orc.exact_sum(x)
    assert ex != 0.0
    cond = float(np.abs(x.astype(np.float64)).sum()) / abs(ex)
    assert cond > 1e8
    comp = prims.reduce_sum(to_dev(x), mode=1)
    naive64 = prims.reduce_sum(to_dev(x.astype(np.float64)))
    err_comp = abs((comp - ex) - exlo)
    err_n64 = abs((naive64 - ex) - exlo)
    assert err_comp <= max(err_n64, 0.5 * np.spacing(abs(ex))), (cond, err_comp, err_n64)
    assert err_comp <= 1e-6 * abs(ex)


def test_f64_sum_special_values_and_exponent_spread(prims, orc):
    """The FP64 sum adds most of each 8-element chunk as exponent-aligned
    int64 mantissas: infinities and NaN must propagate as in FP64, and
    subnormals, wide exponent spreads and huge values must stay within the
    naive bound of the exact sum."""
    rng = np.random.default_rng(31)
    n = 8 * 256 * 64 + 13                      # whole chunks plus a ragged tail
    for pos in (0, 7, 4103, n - 1):
        x = rng.uniform(-1, 1, n)
        x[pos] = np.inf
        assert prims.reduce_sum(to_dev(x)) == np.inf
        x[pos + 1 if pos + 1 < n else pos - 1] = -np.inf
        assert math.isnan(prims.reduce_sum(to_dev(x)))
        x = rng.uniform(-1, 1, n)
        x[pos] = np.nan
        assert math.isnan(prims.reduce_sum(to_dev(x)))
    cases = {
        "subnormal": rng.uniform(-1, 1, n) * 1e-310,
        "spread": rng.uniform(-1, 1, n) * 10.0 ** rng.integers(-300, 300, n),
        "huge": rng.uniform(0.5, 1, n) * 1e300,
        "tiny_and_one": np.where(rng.random(n) < 0.5, 1.0, 1e-20) * rng.choice([-1, 1], n),
        "zeros": np.where(rng.random(n) < 0.5, 0.0, -0.0),
    }
    for name, x in cases.items():
        hi, _ = orc.exact_sum(x)
        a = float(np.abs(x).sum()) if name != "huge" else float(np.abs(x / 1e300).sum()) * 1e300
        got = prims.reduce_sum(to_dev(x))
        assert abs(got - hi) <= naive_bound(n, U64, a) + 1e-300, name
        got_det = prims.reduce_sum(to_dev(x), mode=2)
        assert abs(got_det - hi) <= naive_bound(n, U64, a) + 1e-300, name
    assert prims.reduce_sum(to_dev(np.full(n, 1e308))) == np.inf    # overflows as in FP64
