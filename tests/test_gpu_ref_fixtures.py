"""The CUDA path against RAJA's own results (tests/golden/ref_fixtures.npz).

The fixtures are outputs of RAJA's seq_exec / omp_parallel_for_exec
policies compiled from the unmodified reference headers
(tests/golden/make_ref_fixtures.py).  Parity rules:

  * integer sums, min/max, bit ops, MinLoc/MaxLoc (value and index, ties
    to the lowest index as seq_exec), integer scans of every kind and op,
    histograms: bit for bit;
  * stable sorts (keys and pairs, both directions, against both RAJA
    policies): bit for bit, except that the radix sort orders -0.0 before
    +0.0 while RAJA's comparison sort keeps them in input order (they
    compare equal), so within a run of zero keys values are compared as a
    set;
  * unstable sorts: RAJA's own rule (equal keys, same values per key);
  * floating-point sums: within 2 (n-1) u sum|x| of RAJA's seq result
    (both lie within (n-1) u sum|x| of the exact sum); floating-point scans:
    every prefix within 2 n u sum|x[:i]|; daxpy within 2 u (|y| + |2.5 x|)
    (the GPU fuses a*x+y into one rounding).
"""
import os
import struct

import numpy as np
import pytest

from conftest import to_dev, to_host

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = os.path.join(HERE, "golden", "ref_fixtures.npz")
NP = {"i32": np.int32, "i64": np.int64, "u32": np.uint32, "u64": np.uint64,
      "f32": np.float32, "f64": np.float64}
FMT = {"i32": "i", "i64": "q", "f32": "f", "f64": "d"}
EPS = {"f32": 2.0 ** -24, "f64": 2.0 ** -53}


@pytest.fixture(scope="module")
def fx():
    return dict(np.load(FIX))


def _keys(fx, prefix):
    return sorted(k for k in fx if k.startswith(prefix))


def unpack_reduce(t, raw):
    f = FMT[t]
    bits = t in ("i32", "i64")
    v = struct.unpack("<" + f * 4 + "q" + f + "q" + (f * 2 if bits else ""), raw.tobytes())
    out = {"sum": v[0], "min": v[1], "max": v[2], "minloc": (v[3], v[4]), "maxloc": (v[5], v[6])}
    if bits:
        out["bitor"], out["bitand"] = v[7], v[8]
    return out


@pytest.mark.parametrize("t", ["i32", "i64", "f32", "f64"])
def test_reducers_match_raja(prims, fx, t):
    for key in _keys(fx, f"reduce/{t}/seq/"):
        nm = key.split("/")[3]
        x = fx[f"reduce/{t}/in/{nm}"]
        ref = unpack_reduce(t, fx[key])
        d = to_dev(x)
        got_sum = prims.reduce_sum(d)
        if t in ("i32", "i64"):
            assert got_sum == ref["sum"], key
            assert prims.reduce_bitor(d) == ref["bitor"], key
            assert prims.reduce_bitand(d) == ref["bitand"], key
        else:
            bound = 2 * max(x.size - 1, 1) * EPS[t] * float(np.abs(x.astype(np.float64)).sum())
            assert abs(got_sum - ref["sum"]) <= bound, key
        assert prims.reduce_min(d) == ref["min"], key
        assert prims.reduce_max(d) == ref["max"], key
        v, i = prims.reduce_minloc(d)
        assert (v, i) == ref["minloc"], key
        v, i = prims.reduce_maxloc(d)
        assert (v, i) == ref["maxloc"], key


def test_scans_match_raja(prims, fx):
    n = 0
    for key in _keys(fx, "scan/"):
        parts = key.split("/")
        if parts[2] == "in":
            continue
        t, pol, kind, op, init, nm = parts[1:7]
        x = fx[f"scan/{t}/in/{nm}"]
        ref = fx[key]
        d = to_dev(x)
        iv = 13 if init == "init13" else None
        if kind == "inclusive":
            got = to_host(prims.inclusive_scan(d, op=op))
        elif kind == "exclusive":
            got = to_host(prims.exclusive_scan(d, op=op, init=iv))
        elif kind == "inclusive_inplace":
            got = to_host(prims.inclusive_scan_inplace(d, op=op))
        else:
            got = to_host(prims.exclusive_scan_inplace(d, op=op, init=iv))
        if t in ("i32", "i64"):
            assert np.array_equal(got, ref), key
        else:
            a = np.abs(x.astype(np.float64))
            absp = np.cumsum(a) + abs(iv or 0)
            m = np.arange(1, x.size + 1)
            tol = 2 * m * EPS[t] * absp + 2 * EPS[t] * np.abs(ref.astype(np.float64))
            assert np.all(np.abs(got.astype(np.float64) - ref.astype(np.float64)) <= tol), key
        n += 1
    assert n > 300


def _zero_run_equal(keys, vals, ref_keys, ref_vals):
    """Keys equal as values; values equal position by position except inside
    runs of zero keys (-0.0 / +0.0), where they are equal as sets."""
    if not np.array_equal(keys, ref_keys):
        return False
    z = keys == 0
    return (np.array_equal(vals[~z], ref_vals[~z])
            and np.array_equal(np.sort(vals[z]), np.sort(ref_vals[z])))


def _unstable_equal(keys, vals, ref_keys, ref_vals):
    if not np.array_equal(keys, ref_keys):
        return False
    a, b = np.lexsort((vals, keys)), np.lexsort((ref_vals, ref_keys))
    return np.array_equal(vals[a], ref_vals[b])


def test_sorts_match_raja(prims, fx):
    n = 0
    for key in _keys(fx, "sort/"):
        parts = key.split("/")
        if parts[2] == "in" or not key.endswith("/out") or key.endswith("pairs_out"):
            continue
        t, pol, kind, dr, nn = parts[1:6]
        k = fx[f"sort/{t}/in/{nn}"]
        base = key[: -len("/out")]
        desc = dr == "desc"
        keys_only = to_host(prims.sort(to_dev(k), descending=desc))
        vdt = np.int64 if t in ("i64",) else np.int32
        v = np.arange(k.size, dtype=vdt)
        pk, pv = prims.sort_pairs(to_dev(k), to_dev(v), descending=desc)
        pk, pv = to_host(pk), to_host(pv).astype(np.int32)
        rk, rv = fx[base + "/pairs_out"], fx[base + "/pairs_vout"]
        if kind == "stable_sort":
            if t[0] == "f":
                assert _zero_run_equal(keys_only, keys_only, fx[key], fx[key]), key
                assert _zero_run_equal(pk, pv, rk, rv), key
            else:
                assert np.array_equal(keys_only, fx[key]), key
                assert np.array_equal(pk, rk) and np.array_equal(pv, rv), key
        else:
            assert np.array_equal(keys_only, fx[key]), key
            assert _unstable_equal(pk, pv, rk, rv), key
        n += 1
    assert n == 240


def test_histogram_and_daxpy_match_raja(prims, fx):
    for nb in (256, 65536):
        b = fx[f"hist/in/bins{nb}"]
        got = to_host(prims.histogram(to_dev(b), nb))
        for pol in ("seq", "omp"):
            assert np.array_equal(got, fx[f"hist/{pol}/bins{nb}/out"]), (nb, pol)
    x, y = fx["daxpy/x"], fx["daxpy/y"]
    dy = to_dev(y.copy())
    prims.forall_axpy(2.5, to_dev(x), dy)
    got = to_host(dy)
    for pol in ("seq", "omp"):
        ref = fx[f"daxpy/{pol}/out"]
        # one rounding (fused) against two (product, then sum)
        tol = 2 * EPS["f64"] * (np.abs(y) + 2.5 * np.abs(x))
        assert np.all(np.abs(got - ref) <= tol), pol
