"""Scans through the C ABI vs the oracle: bit-exact for integers and for
min/max; floating-point sums within stated bounds of double-double prefix
sums."""
import os

import numpy as np
import pytest

from conftest import to_dev, to_host

pytestmark = pytest.mark.gpu

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
# tile boundaries: 64 KB tiles hold 16384 elements of a 4-byte type and 8192
# of an 8-byte type; the compensated sums use 32 KB tiles (8192 / 4096)
SIZES = [0, 1, 2, 31, 32, 33, 4095, 4096, 4097, 8191, 8192, 8193, 16383, 16384, 16385,
         49153, 65536 + 7, (1 << 20) + 3]


def test_golden_scan(prims):
    g = np.load(os.path.join(G, "scan.npz"))
    np.testing.assert_array_equal(to_host(prims.inclusive_scan(to_dev(g["a"]))), g["a_incl"])
    np.testing.assert_array_equal(to_host(prims.exclusive_scan(to_dev(g["a"]))), g["a_excl"])
    np.testing.assert_array_equal(to_host(prims.exclusive_scan(to_dev(g["b"]), init=7)), g["b_excl7"])
    np.testing.assert_array_equal(to_host(prims.inclusive_scan(to_dev(g["iota"]), op="min")), g["iota_min"])
    np.testing.assert_array_equal(to_host(prims.inclusive_scan(to_dev(g["iota"]), op="max")), g["iota_max"])
    np.testing.assert_array_equal(to_host(prims.inclusive_scan(to_dev(g["rev"]), op="min")), g["rev_min"])


def _input(dt, n, seed):
    rng = np.random.default_rng(seed)
    if np.dtype(dt).kind == "u":
        return rng.integers(0, np.iinfo(dt).max, n, dtype=np.uint64).astype(dt)
    if np.dtype(dt).kind == "i":
        return rng.integers(np.iinfo(dt).min // 2, np.iinfo(dt).max // 2, n, dtype=np.int64).astype(dt)
    return rng.uniform(-1, 1, n).astype(dt)


@pytest.mark.parametrize("dt", [np.int32, np.int64, np.uint32, np.uint64])
@pytest.mark.parametrize("op", ["plus", "minimum", "maximum"])
def test_integer_scans_bit_exact(prims, orc, dt, op):
    for i, n in enumerate(SIZES):
        x = _input(dt, n, 10 * i + 1)
        d = to_dev(x)
        np.testing.assert_array_equal(to_host(prims.inclusive_scan(d, op=op)),
                                      orc.scan(x, op), err_msg=f"n={n}")
        init = x[0] if n else dt(5)
        np.testing.assert_array_equal(to_host(prims.exclusive_scan(d, op=op, init=init)),
                                      orc.scan(x, op, exclusive=True, init=init), err_msg=f"n={n}")


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("op", ["minimum", "maximum"])
def test_float_minmax_scans_bit_exact(prims, orc, dt, op):
    for i, n in enumerate(SIZES):
        x = _input(dt, n, 10 * i + 2)
        if n > 10:
            x[5] = np.inf
            x[7] = -np.inf
        d = to_dev(x)
        np.testing.assert_array_equal(to_host(prims.inclusive_scan(d, op=op)), orc.scan(x, op))
        np.testing.assert_array_equal(to_host(prims.exclusive_scan(d, op=op, init=0.25)),
                                      orc.scan(x, op, exclusive=True, init=0.25))


def test_inplace_and_misaligned(prims, orc):
    import torch
    for n in (4097, 100003):
        x = _input(np.int32, n, n)
        d = to_dev(x)
        prims.inclusive_scan_inplace(d)
        np.testing.assert_array_equal(to_host(d), orc.scan(x, "plus"))
        d = to_dev(x)
        prims.exclusive_scan_inplace(d, init=3)
        np.testing.assert_array_equal(to_host(d), orc.scan(x, "plus", exclusive=True, init=3))
        big = to_dev(x)
        for off in (1, 2, 3):
            out = torch.empty(n - off, dtype=torch.int32, device="cuda")
            prims.inclusive_scan(big[off:], out=out)
            np.testing.assert_array_equal(to_host(out), orc.scan(x[off:], "plus"))


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_float_sum_scans_within_bounds(prims, orc, dt):
    u = 2.0 ** -24 if dt == np.float32 else 2.0 ** -53
    for i, n in enumerate(SIZES[1:]):
        x = np.random.default_rng(i).uniform(0, 1, n).astype(dt)
        ref = orc.dd_scan_f32(x) if dt == np.float32 else np.cumsum(x.astype(np.longdouble)).astype(np.float64)
        absp = np.cumsum(np.abs(x.astype(np.float64)))
        got = to_host(prims.inclusive_scan(to_dev(x))).astype(np.float64)
        # tree order: error <= (log2(n) + items per thread + 2) u sum|x| per prefix
        k = np.log2(max(n, 2)) + 32
        assert np.all(np.abs(got - ref) <= k * u * absp + 1e-300)
        got = to_host(prims.inclusive_scan(to_dev(x), mode=1)).astype(np.float64)
        # compensated: the output rounding (u |prefix|) dominates
        assert np.all(np.abs(got - ref) <= 2 * u * np.abs(ref) + 1e-6 * u * absp + 1e-300)
        got = to_host(prims.exclusive_scan(to_dev(x), init=1.5, mode=1)).astype(np.float64)
        exp = np.concatenate([[1.5], 1.5 + ref[:-1]])
        assert np.all(np.abs(got - exp) <= 2 * u * np.abs(exp) + 1e-6 * u * (absp + 1.5) + 1e-300)


def test_leading_negative_zero_survives(prims):
    import torch
    x = torch.tensor([-0.0, -0.0, 1.0], dtype=torch.float32, device="cuda")
    r = prims.inclusive_scan(x)
    assert str(r[0].item()) == "-0.0" and str(r[1].item()) == "-0.0"
