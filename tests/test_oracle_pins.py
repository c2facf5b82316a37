"""Pin the oracle against the known answers of RAJA's own test suite.

RAJA cannot be built in this environment (its camp/BLT submodules are
empty), so the CPU restatement in oracle/ is pinned against the checks the
reference tests perform, restated here with fixed seeds:

  test/functional/forall/reduce-basic/tests/test-forall-basic-Reduce*.hpp
  test/functional/scan/tests/test-scan-{Inclusive,Exclusive}*.hpp
  test/unit/algorithm/tests/test-algorithm-{sort,stable-sort}*.hpp
  test/functional/forall/multi-reduce-basic/tests/test-forall-basic-MultiReduce.hpp

and against independent numpy / math.fsum computations.
"""
import math

import numpy as np
import pytest

# Segments of the reduce-basic tests: ranges (0,28), (3,642), (0,2057);
# strided (0,188,2), (3,1029,3); and a random list segment.
def _segments(rng):
    segs = [np.arange(0, 28), np.arange(3, 642), np.arange(0, 2057),
            np.arange(0, 188, 2), np.arange(3, 1029, 3)]
    last = 10567
    keep = [i for i in range(last) if rng.integers(0, last) > i]  # i < randval
    segs.append(np.array(keep if keep else [0]))
    return segs


DTYPES = [np.int32, np.int64, np.float32, np.float64]


@pytest.mark.parametrize("dt", DTYPES)
def test_reduce_sum_known_answers(orc, dt):
    rng = np.random.default_rng(1)
    for seg in _segments(rng):
        data = rng.integers(0, 100, seg[-1] + 1).astype(dt)  # rand() % modval
        vals = np.ascontiguousarray(data[seg])
        ref_sum = dt(0)
        for v in vals:
            ref_sum = dt(ref_sum + v)
        assert orc.reduce_sum(vals, 0) == ref_sum
        assert orc.reduce_sum(vals, 2) == ref_sum + 2
        # reset + two loops accumulate twice
        assert orc.reduce_sum(np.concatenate([vals, vals]), 0) == 2 * ref_sum


@pytest.mark.parametrize("dt", DTYPES)
def test_reduce_minloc_maxloc_known_answers(orc, dt):
    rng = np.random.default_rng(2)
    modval = 100
    for seg in _segments(rng):
        idx_len = len(seg)
        data = rng.integers(0, modval, seg[-1] + 1).astype(dt)
        loc_idx = seg[idx_len * 2 // 3]
        # MinLoc: plant -modval
        d = data.copy()
        d[loc_idx] = -modval
        vals = np.ascontiguousarray(d[seg])
        ref_min, ref_loc = dt(modval + 1), -1
        for i, v in enumerate(vals):
            if v < ref_min:
                ref_min, ref_loc = v, int(seg[i])
        v, l = orc.reduce_minloc(vals, init_val=-modval, init_loc=-1)
        assert (v, l) == (-modval, -1)        # init ties with the data: init wins
        v, l = orc.reduce_minloc(vals, init_val=modval + 1, init_loc=-1)
        assert v == ref_min and int(seg[l]) == ref_loc
        # MaxLoc: plant modval+1
        d = data.copy()
        d[loc_idx] = modval + 1
        vals = np.ascontiguousarray(d[seg])
        ref_max, ref_loc = dt(-modval), -1
        for i, v in enumerate(vals):
            if v > ref_max:
                ref_max, ref_loc = v, int(seg[i])
        v, l = orc.reduce_maxloc(vals, init_val=modval + 1, init_loc=-1)
        assert (v, l) == (modval + 1, -1)
        v, l = orc.reduce_maxloc(vals, init_val=-modval, init_loc=-1)
        assert v == ref_max and int(seg[l]) == ref_loc


@pytest.mark.parametrize("dt", [np.int32, np.int64, np.uint32, np.uint64])
def test_reduce_bit_known_answers(orc, dt):
    rng = np.random.default_rng(3)
    for seg in _segments(rng):
        nines = np.full(len(seg), 9, dtype=dt)
        assert orc.reduce_bitor(nines, 5) == 13              # 9 | 5
        data = rng.integers(0, 100, len(seg)).astype(dt)
        ref_or = 0
        for v in data:
            ref_or |= int(v)
        assert orc.reduce_bitor(data, 0) == ref_or
        assert orc.reduce_bitor(data, 2) == ref_or | 2
        ref_and = int(np.iinfo(dt).max) if np.dtype(dt).kind == "u" else -1
        for v in data:
            ref_and &= int(v)
        assert int(orc.reduce_bitand(data)) == ref_and


def test_min_max_first_wins(orc):
    # operators::minimum keeps lhs unless rhs < lhs: the first extreme wins,
    # which shows on signed zeros and on repeated extremes.
    x = np.array([0.0, -0.0, 3.0, -1.0, -1.0, 5.0, 5.0], dtype=np.float64)
    assert orc.reduce_minloc(x) == (-1.0, 3)
    assert orc.reduce_maxloc(x) == (5.0, 5)
    z = np.array([0.0, -0.0], dtype=np.float64)
    assert math.copysign(1.0, orc.reduce_min(z)) == 1.0
    z = np.array([-0.0, 0.0], dtype=np.float64)
    assert math.copysign(1.0, orc.reduce_min(z)) == -1.0
    # empty input: the identity (limits max, -1)
    e = np.zeros(0, dtype=np.float32)
    assert orc.reduce_minloc(e) == (float(np.finfo(np.float32).max), -1)
    assert orc.reduce_maxloc(e) == (float(-np.finfo(np.float32).max), -1)


SCAN_OPS = ["plus", "minimum", "maximum"]
SCAN_TYPES = [np.int32, np.float32, np.float64]


def _identity(op, dt):
    if op == "plus":
        return dt(0)
    if np.dtype(dt).kind == "f":
        return dt(np.finfo(dt).max if op == "minimum" else -np.finfo(dt).max)
    return dt(np.iinfo(dt).max if op == "minimum" else np.iinfo(dt).min)


def _apply(op, a, b):
    if op == "plus":
        return a + b
    if op == "minimum":
        return b if b < a else a
    return b if a < b else a


@pytest.mark.parametrize("op", SCAN_OPS)
@pytest.mark.parametrize("dt", SCAN_TYPES)
@pytest.mark.parametrize("n", [0, 357, 32000])
@pytest.mark.parametrize("parallel", [False, True])
def test_scan_known_answers(orc, op, dt, n, parallel):
    if op == "plus" and dt == np.float32 and parallel:
        pytest.skip("the reference disables plus<float> scans (precision)")
    x = np.arange(1, n + 1).astype(dt)                       # std::iota(.., 1)
    # check_inclusive: running OP from OP::identity()
    acc = _identity(op, dt)
    exp = np.empty(n, dtype=dt)
    for i in range(n):
        acc = dt(_apply(op, acc, x[i]))
        exp[i] = acc
    got = orc.scan(x, op, exclusive=False, parallel=parallel)
    np.testing.assert_array_equal(got, exp)
    # in-place form
    y = x.copy()
    orc.scan(y, op, exclusive=False, parallel=parallel, out=y)
    np.testing.assert_array_equal(y, exp)
    # check_exclusive with identity and with the non-identity offsets 13/15/2
    for init in (_identity(op, dt), dt({0: 13, 357: 15, 32000: 2}[n])):
        acc = dt(init)
        exp = np.empty(n, dtype=dt)
        for i in range(n):
            exp[i] = acc
            acc = dt(_apply(op, acc, x[i]))
        got = orc.scan(x, op, exclusive=True, init=init, parallel=parallel)
        np.testing.assert_array_equal(got, exp)


SORT_KEYS = [np.int64, np.int32, np.float64, np.uint32, np.uint64, np.float32]


@pytest.mark.parametrize("kt", SORT_KEYS)
@pytest.mark.parametrize("max_n", [0, 1, 10, 100, 1000, 10000])
@pytest.mark.parametrize("parallel", [False, True])
def test_sort_known_answers(orc, kt, max_n, parallel):
    # mt19937(seed) size in [(MaxN+1)/2, MaxN], keys uniform in [-N, N]
    rng = np.random.default_rng(max_n + 7)
    n = int(rng.integers((max_n + 1) // 2, max_n + 1)) if max_n else 0
    if np.dtype(kt).kind == "u":
        keys = rng.integers(0, 2 * n + 1, n).astype(kt)
    else:
        keys = rng.integers(-n, n + 1, n).astype(kt)
    vals = np.arange(n, dtype=np.int64)
    for desc in (False, True):
        got = orc.sort(keys, descending=desc, parallel=parallel)
        exp = np.sort(keys, kind="stable")
        if desc:
            exp = exp[::-1]
        np.testing.assert_array_equal(got, exp)
        # stable pairs: exact; equal keys keep input order
        pk = keys.astype(np.float64) if kt == np.float64 else keys
        name_ok = {np.dtype(np.float64): np.int64, np.dtype(np.int64): np.int64,
                   np.dtype(np.uint64): np.int64}
        vt = name_ok.get(np.dtype(kt), np.int32)
        k2, v2 = orc.sort_pairs(pk, vals.astype(vt), descending=desc, parallel=parallel)
        order = np.argsort(-pk.astype(np.float64) if desc else pk, kind="stable") if kt != np.uint64 \
            else (np.argsort(pk, kind="stable")[::-1] if desc else np.argsort(pk, kind="stable"))
        if kt == np.uint64 and desc:
            # stable descending: reverse of the ascending order within groups
            order = np.lexsort((np.arange(n), -np.argsort(np.argsort(pk, kind="stable"))))
            order = np.array(sorted(range(n), key=lambda i: (-int(pk[i]), i)), dtype=np.int64)
        np.testing.assert_array_equal(k2, pk[order])
        np.testing.assert_array_equal(v2, vals[order].astype(vt))


@pytest.mark.parametrize("nbins", [1, 7, 256, 65536])
def test_multireduce_histogram_known_answers(orc, nbins):
    rng = np.random.default_rng(nbins)
    x = rng.integers(0, nbins, 12345).astype(np.int32)
    exp = np.bincount(x, minlength=nbins).astype(np.uint64)
    np.testing.assert_array_equal(orc.histogram(x, nbins), exp)
    np.testing.assert_array_equal(orc.histogram(x, nbins, parallel=True), exp)
    # values outside [0, nbins) are not counted
    y = np.concatenate([x, np.array([-1, nbins, nbins + 5], dtype=np.int32)])
    np.testing.assert_array_equal(orc.histogram(y, nbins), exp)


def test_exact_accumulator_matches_fsum(orc):
    rng = np.random.default_rng(5)
    for dt in (np.float32, np.float64):
        x = (rng.choice([-1.0, 1.0], 20000) * np.exp(rng.normal(0, 6, 20000))).astype(dt)
        hi, lo = orc.exact_sum(x)
        assert hi == math.fsum(x.astype(np.float64).tolist())
        # hi + lo carries more than double precision: check against fractions
        from fractions import Fraction
        exact = sum(Fraction(float(v)) for v in x.astype(np.float64))
        assert abs(Fraction(hi) + Fraction(lo) - exact) <= abs(exact) * Fraction(1, 2 ** 100) + Fraction(1, 2 ** 1070)
    # dot with exact products
    x = rng.normal(size=3000)
    y = rng.normal(size=3000)
    hi, lo = orc.exact_dot(x, y)
    from fractions import Fraction
    exact = sum(Fraction(float(a)) * Fraction(float(b)) for a, b in zip(x, y))
    assert abs(Fraction(hi) + Fraction(lo) - exact) <= abs(exact) * Fraction(1, 2 ** 100)


def test_seq_fp_sum_is_left_fold(orc):
    # seq ReduceSum: init + (((0 + x0) + x1) + ...) in the element type
    rng = np.random.default_rng(6)
    x = rng.uniform(-1, 1, 5000).astype(np.float32)
    acc = np.float32(0)
    for v in x:
        acc = np.float32(acc + v)
    assert orc.reduce_sum(x, 0.5) == np.float32(np.float32(0.5) + acc)
    # dot: products rounded, then added (no contraction)
    y = rng.uniform(-1, 1, 5000).astype(np.float32)
    acc = np.float32(0)
    for a, b in zip(x, y):
        acc = np.float32(acc + np.float32(a * b))
    assert orc.dot(x, y) == acc


def test_omp_paths_agree_with_seq(orc):
    rng = np.random.default_rng(8)
    xi = rng.integers(0, 1024, 100003).astype(np.int64)
    np.testing.assert_array_equal(orc.scan(xi, "plus", exclusive=True, parallel=True),
                                  orc.scan(xi, "plus", exclusive=True, parallel=False))
    xf = rng.uniform(-1, 1, 100003)
    assert orc.reduce_minloc(xf, parallel=True) == orc.reduce_minloc(xf)
    assert orc.reduce_maxloc(xf, parallel=True) == orc.reduce_maxloc(xf)
    assert abs(orc.reduce_sum(xf, parallel=True) - math.fsum(xf.tolist())) < 1e-9
    k = rng.integers(0, 2 ** 32, 50001, dtype=np.uint64).astype(np.uint32)
    np.testing.assert_array_equal(orc.sort(k, parallel=True), np.sort(k))
    y = rng.uniform(-1, 1, 100003)
    y2 = y.copy()
    orc.axpy(2.5, xf, y, parallel=True)
    orc.axpy(2.5, xf, y2, parallel=False)
    np.testing.assert_array_equal(y, y2)


def test_oracle_multi_reduce_vs_numpy_at():
    """The oracle's MultiReduce restatement against numpy's unbuffered
    ufunc.at (integers: order does not matter), out-of-range bins skipped."""
    import oracle
    rng = np.random.default_rng(41)
    n, nbins = 20000, 37
    bins = rng.integers(-2, nbins + 2, n).astype(np.int32)
    ok = (bins >= 0) & (bins < nbins)
    for dt in (np.int32, np.int64, np.uint32, np.uint64):
        vals = rng.integers(0, 1 << 30, n).astype(dt)
        for op, uf, init in (("sum", np.add, 0), ("min", np.minimum, np.iinfo(dt).max),
                             ("max", np.maximum, np.iinfo(dt).min), ("bitor", np.bitwise_or, 0),
                             ("bitand", np.bitwise_and, np.iinfo(dt).max)):
            ref = np.full(nbins, init, dtype=dt)
            uf.at(ref, bins[ok], vals[ok])
            got = oracle.multi_reduce(op, bins, vals, np.full(nbins, init, dtype=dt))
            np.testing.assert_array_equal(got, ref, err_msg=f"{op} {dt}")
    # floats: min keeps the first of equal values and skips NaN
    v = np.array([2.0, np.nan, 1.0, 1.0, -0.0, 0.0])
    b = np.array([0, 0, 0, 1, 2, 2], np.int32)
    got = oracle.multi_reduce("min", b, v, np.full(3, np.inf))
    assert got[0] == 1.0 and got[1] == 1.0 and np.signbit(got[2])
