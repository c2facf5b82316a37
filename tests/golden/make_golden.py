"""Generate the golden fixtures in tests/golden/*.npz.

Each fixture holds seeded inputs (numpy default_rng, platform independent)
and expected outputs computed with numpy and math.fsum -- an implementation
independent of both the oracle and the CUDA library.  The shapes follow the
reference test suite and the benchmark configurations at small sizes:

  reduce.npz     f64/f32 uniform[-1,1) sums, dots, min/max(loc) with planted
                 ties, int32 rand()%100 sums and bit reductions
  scan.npz       int32 uniform[0,16) and int64 uniform[0,1024) inclusive /
                 exclusive sums; iota min/max scans
  sort.npz       u32 full-range keys with int32 index values, f32 normal keys,
                 u64 keys, keys uniform in [-N, N] (duplicates), descending
  histogram.npz  Zipf(1.1) int32 values binned into 256 and 65536 bins
  axpy.npz       daxpy y += 2.5 x

Run:  python tests/golden/make_golden.py
"""
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def zipf_bins(rng, n, nbins, s=1.1):
    """Zipf(s) over bins 0..nbins-1 by inverse CDF (support clipped)."""
    w = 1.0 / np.arange(1, nbins + 1, dtype=np.float64) ** s
    cdf = np.cumsum(w)
    cdf /= cdf[-1]
    return np.searchsorted(cdf, rng.random(n), side="right").clip(0, nbins - 1).astype(np.int32)


def reduce_fixture():
    rng = np.random.default_rng(0)
    n = 4097
    x64 = rng.uniform(-1, 1, n)
    y64 = rng.uniform(-1, 1, n)
    x32 = rng.uniform(-1, 1, n).astype(np.float32)
    y32 = rng.uniform(-1, 1, n).astype(np.float32)
    # planted ties for min/max loc: several copies of the extremes
    t32 = rng.integers(0, 8, n).astype(np.float32)
    i32 = rng.integers(0, 100, n).astype(np.int32)
    return dict(
        x64=x64, y64=y64, x32=x32, y32=y32, t32=t32, i32=i32,
        sum64=math.fsum(x64.tolist()), sum32=math.fsum(x32.astype(np.float64).tolist()),
        dot64=math.fsum((x64 * y64).tolist()),
        dot32=math.fsum((x32.astype(np.float64) * y32.astype(np.float64)).tolist()),
        abs64=math.fsum(np.abs(x64).tolist()), abs32=math.fsum(np.abs(x32.astype(np.float64)).tolist()),
        min64=x64.min(), max64=x64.max(), argmin64=int(np.argmin(x64)), argmax64=int(np.argmax(x64)),
        min_t32=t32.min(), argmin_t32=int(np.argmin(t32)), max_t32=t32.max(), argmax_t32=int(np.argmax(t32)),
        sum_i32=int(i32.astype(np.int64).sum()),
        or_i32=int(np.bitwise_or.reduce(i32)), and_i32=int(np.bitwise_and.reduce(i32)),
    )


def scan_fixture():
    rng = np.random.default_rng(1)
    n = 10007
    a = rng.integers(0, 16, n).astype(np.int32)
    b = rng.integers(0, 1024, n).astype(np.int64)
    iota = np.arange(1, 32001, dtype=np.int32)
    return dict(
        a=a, a_incl=np.cumsum(a, dtype=np.int64).astype(np.int32),
        a_excl=np.concatenate([[0], np.cumsum(a, dtype=np.int64)[:-1]]).astype(np.int32),
        b=b, b_excl7=np.concatenate([[7], 7 + np.cumsum(b)[:-1]]).astype(np.int64),
        iota=iota, iota_min=np.minimum.accumulate(iota), iota_max=np.maximum.accumulate(iota),
        rev=iota[::-1].copy(), rev_min=np.minimum.accumulate(iota[::-1]),
    )


def sort_fixture():
    rng = np.random.default_rng(2)
    n = 10007
    ku = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    idx = np.arange(n, dtype=np.int32)
    order_u = np.argsort(ku, kind="stable")
    kf = rng.normal(0, 1, n).astype(np.float32)
    order_f = np.argsort(kf, kind="stable")
    k64 = rng.integers(0, 2 ** 63, n, dtype=np.uint64) * np.uint64(2) + rng.integers(0, 2, n, dtype=np.uint64)
    kd = rng.integers(-n, n + 1, n).astype(np.int32)             # duplicates
    order_d = np.argsort(kd, kind="stable")
    order_d_desc = np.array(sorted(range(n), key=lambda i: (-int(kd[i]), i)), dtype=np.int64)
    return dict(
        ku=ku, ku_sorted=ku[order_u], ku_perm=idx[order_u],
        kf=kf, kf_sorted=kf[order_f], kf_perm=idx[order_f],
        k64=k64, k64_sorted=np.sort(k64), k64_desc=np.sort(k64)[::-1].copy(),
        kd=kd, kd_sorted=kd[order_d], kd_perm=idx[order_d],
        kd_desc=kd[order_d_desc], kd_desc_perm=idx[order_d_desc],
    )


def histogram_fixture():
    rng = np.random.default_rng(3)
    n = 100003
    z256 = zipf_bins(rng, n, 256)
    z64k = zipf_bins(rng, n, 65536)
    return dict(z256=z256, h256=np.bincount(z256, minlength=256).astype(np.int64),
                z64k=z64k, h64k=np.bincount(z64k, minlength=65536).astype(np.int64))


def axpy_fixture():
    rng = np.random.default_rng(4)
    n = 4099
    x = rng.uniform(-1, 1, n)
    y = rng.uniform(-1, 1, n)
    return dict(x=x, y=y, a=2.5, y_out=y + 2.5 * x)


def main():
    for name, fn in [("reduce", reduce_fixture), ("scan", scan_fixture), ("sort", sort_fixture),
                     ("histogram", histogram_fixture), ("axpy", axpy_fixture)]:
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **fn())
        print(path, os.path.getsize(path))


if __name__ == "__main__":
    main()
