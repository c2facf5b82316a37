"""Binned reductions (MultiReduce{Sum,Min,Max,BitOr,BitAnd}) through the C
ABI against the oracle's seq restatement: integer, bit, min and max results
bit-exact; floating-point sums within a stated bound per bin."""
import numpy as np
import pytest

from conftest import to_dev, to_host

pytestmark = pytest.mark.gpu

TYPES = [np.int32, np.int64, np.uint32, np.uint64, np.float32, np.float64]
U = {np.dtype(np.float32): 2.0 ** -24, np.dtype(np.float64): 2.0 ** -53}


def _vals(dt, n, rng):
    dt = np.dtype(dt)
    if dt.kind == "f":
        return rng.normal(0, 100, n).astype(dt)
    info = np.iinfo(dt)
    if dt.itemsize == 8:
        return rng.integers(0, 2 ** 64, n, dtype=np.uint64).view(dt) if dt.kind == "i" else \
            rng.integers(0, 2 ** 64, n, dtype=np.uint64)
    return rng.integers(info.min, info.max, n, dtype=np.int64).astype(dt)


def _identity(op, dt):
    dt = np.dtype(dt)
    if op in ("sum", "bitor"):
        return dt.type(0)
    if op == "bitand":
        return np.array(-1).astype(np.int64).astype(dt) if dt.kind == "i" else dt.type(np.iinfo(dt).max)
    if dt.kind == "f":
        return dt.type(np.finfo(dt).max if op == "min" else -np.finfo(dt).max)
    return dt.type(np.iinfo(dt).max if op == "min" else np.iinfo(dt).min)


def _check(prims, orc, op, dt, n, nbins, seed, init=None):
    rng = np.random.default_rng(seed)
    bins = rng.integers(-3, nbins + 3, n).astype(np.int32)        # some out of range
    vals = _vals(dt, n, rng)
    start = np.full(nbins, _identity(op, dt) if init is None else init, dtype=dt)
    got = to_host(prims.multi_reduce(op, to_dev(bins), to_dev(vals), out=to_dev(start.copy())))
    ref = orc.multi_reduce(op, bins, vals, start.copy())
    if np.dtype(dt).kind == "f" and op == "sum":
        absum = orc.multi_reduce("sum", bins, np.abs(vals), np.abs(start.copy()))
        cnt = np.bincount(bins[(bins >= 0) & (bins < nbins)], minlength=nbins)
        bound = (cnt + 1) * U[np.dtype(dt)] * absum + 1e-30
        assert np.all(np.abs(got.astype(np.float64) - ref) <= bound), (op, dt, n, nbins)
    else:
        np.testing.assert_array_equal(got, ref, err_msg=f"{op} {dt} n={n} nbins={nbins}")


@pytest.mark.parametrize("dt", TYPES)
@pytest.mark.parametrize("op", ["sum", "min", "max"])
def test_multi_reduce_matches_seq(prims, orc, op, dt):
    for i, (n, nbins) in enumerate(((0, 5), (1, 1), (100003, 1), (100003, 7), (100003, 256),
                                    (1 << 20, 5000), (1 << 20, 65536), (300007, 200000))):
        _check(prims, orc, op, dt, n, nbins, 10 * i + 1)


@pytest.mark.parametrize("dt", [np.int32, np.int64, np.uint32, np.uint64])
@pytest.mark.parametrize("op", ["bitor", "bitand"])
def test_multi_reduce_bits(prims, orc, op, dt):
    for i, (n, nbins) in enumerate(((100003, 3), (1 << 20, 4096), (300007, 150000))):
        _check(prims, orc, op, dt, n, nbins, 20 * i + 3)


def test_multi_reduce_init_values_and_nan(prims, orc):
    rng = np.random.default_rng(5)
    _check(prims, orc, "sum", np.int64, 100003, 100, 1, init=np.int64(5))
    _check(prims, orc, "min", np.float64, 100003, 100, 2, init=np.float64(-50.0))
    _check(prims, orc, "max", np.uint32, 100003, 100, 3, init=np.uint32(7))
    # NaN values never enter min / max (operator< rule); sums propagate them
    n, nbins = 100003, 64
    bins = rng.integers(0, nbins, n).astype(np.int32)
    vals = rng.normal(0, 1, n)
    vals[rng.integers(0, n, 500)] = np.nan
    for op in ("min", "max"):
        start = np.full(nbins, _identity(op, np.float64))
        got = to_host(prims.multi_reduce(op, to_dev(bins), to_dev(vals), out=to_dev(start.copy())))
        np.testing.assert_array_equal(got, orc.multi_reduce(op, bins, vals, start.copy()))
    got = to_host(prims.multi_reduce("sum", to_dev(bins), to_dev(vals), nbins))
    ref = orc.multi_reduce("sum", bins, vals, np.zeros(nbins))
    assert np.array_equal(np.isnan(got), np.isnan(ref))


def test_multi_reduce_default_identity_and_errors(prims):
    import torch
    bins = torch.tensor([0, 1, 1, 3], dtype=torch.int32, device="cuda")
    vals = torch.tensor([4, -2, 9, 1], dtype=torch.int32, device="cuda")
    assert prims.multi_reduce("min", bins, vals, 4).tolist() == [4, -2, 2 ** 31 - 1, 1]
    assert prims.multi_reduce("max", bins, vals, 4).tolist() == [4, 9, -2 ** 31, 1]
    assert prims.multi_reduce("sum", bins, vals, 4).tolist() == [4, 7, 0, 1]
    u = vals.view(torch.uint32)
    got = prims.multi_reduce("bitand", bins, u, 4).view(torch.int32).tolist()
    assert got == [4, -2 & 9, -1, 1]
    with pytest.raises(TypeError):
        prims.multi_reduce("bitor", bins, vals.float(), 4)
    with pytest.raises(Exception):
        prims.multi_reduce("sum", bins, vals, 0)
