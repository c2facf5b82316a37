"""The exact reference that bench.py's accuracy leg measures against:
integer-limb sums and prefix sums, checked against math.fsum / fractions on
the CPU (the same torch code runs on the device in the bench)."""
import math
from fractions import Fraction

import numpy as np
import pytest
import torch

import bench


def _illcond(rng, n):
    sign = rng.choice([-1.0, 1.0], n)
    return (sign * np.clip(np.exp(rng.normal(0, 6, n)), 1e-8, 1e8)).astype(np.float32)


@pytest.mark.parametrize("n", [1, 7, 1000, 50000])
def test_exact_sum_matches_fsum(n):
    rng = np.random.default_rng(n)
    x = _illcond(rng, n)
    hi, lo = bench.exact_sum(torch.from_numpy(x))
    exact = sum(Fraction(float(v)) for v in x)
    assert hi == float(exact)                       # correctly rounded
    assert lo == float(exact - Fraction(hi))
    assert hi == math.fsum(x.astype(np.float64))


def test_exact_sum_cancellation_and_doubles():
    rng = np.random.default_rng(1)
    x = _illcond(rng, 20000)
    head, _ = bench.exact_sum(torch.from_numpy(x[:-1]))
    x[-1] = np.float32(-head)                       # cancel to the FP32 rounding residue
    hi, lo = bench.exact_sum(torch.from_numpy(x))
    exact = sum(Fraction(float(v)) for v in x)
    assert hi == float(exact) and abs(exact) < 1e-5 * np.abs(x.astype(np.float64)).sum()
    # products of two floats are exact in double: the dot reference
    y = _illcond(rng, 20000)
    p = x.astype(np.float64) * y.astype(np.float64)
    dh, _ = bench.exact_sum(torch.from_numpy(p))
    assert dh == float(sum(Fraction(float(a)) * Fraction(float(b)) for a, b in zip(x, y)))
    assert bench.exact_sum(torch.zeros(5)) == (0.0, 0.0)


def test_exact_prefix_matches_fractions():
    rng = np.random.default_rng(2)
    x = _illcond(rng, 3000)
    got = bench.exact_prefix_f64(torch.from_numpy(x)).numpy()
    run = Fraction(0)
    for i, v in enumerate(x):
        run += Fraction(float(v))
        assert abs(got[i] - float(run)) <= 4 * np.spacing(abs(float(run))) + 1e-300, i
