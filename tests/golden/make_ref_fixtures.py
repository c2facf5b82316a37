"""Generate tests/golden/ref_fixtures.npz from RAJA itself.

Runs oracle/_ref/ref_driver -- RAJA's own seq_exec / omp_parallel_for_exec
policies, reducers, scans, sorts, MultiReduceSum and WorkGroup, compiled
from the unmodified reference headers (oracle/refbuild/build_ref.py) -- on
seeded inputs and stores inputs and outputs together.  The fixtures pin the
oracle (tests/test_ref_fixtures.py), the compat front-end's host policies
and the GPU path (tests/test_gpu_ref_fixtures.py) to RAJA's actual results.

Run here, where the reference tree is available:

    python tests/golden/make_ref_fixtures.py [--ref /path/to/RAJA]

The OpenMP cases run with OMP_NUM_THREADS=4 (stored in the file): RAJA's
OpenMP scan splits the input into one block per thread, so floating-point
results depend on the thread count.  Key layout: inputs once per case as
"<case>/<type>/in/<input>", results as "<case>/<type>/<policy>/.../out"
(sorts add "pairs_out" and "pairs_vout", the values being 0..n-1).
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
OUT = os.path.join(HERE, "ref_fixtures.npz")
OMP_THREADS = 4

NP = {"i32": np.int32, "i64": np.int64, "u32": np.uint32, "u64": np.uint64,
      "f32": np.float32, "f64": np.float64}


class Driver:
    def __init__(self, exe: str):
        self.exe = exe
        self.tmp = tempfile.mkdtemp(prefix="ref_fixtures_")
        self.env = dict(os.environ, OMP_NUM_THREADS=str(OMP_THREADS), OMP_PROC_BIND="false")
        self.k = 0

    def path(self, arr=None) -> str:
        self.k += 1
        p = os.path.join(self.tmp, f"a{self.k}.bin")
        if arr is not None:
            np.ascontiguousarray(arr).tofile(p)
        return p

    def run(self, *args):
        subprocess.run([self.exe] + [str(a) for a in args], check=True, env=self.env)


def reduce_inputs(rng):
    """RAJA's reduce-basic shapes: rand() % 100 data over segments of 1, 28,
    639, 2057 and 10567 elements (many ties), with a planted minimum of -100
    and maximum of 200 at idx_len*2/3 and idx_len/3 in a second copy; plus
    uniform[-1,1) floats."""
    out = []
    for n in (1, 28, 639, 2057, 10567):
        x = rng.integers(0, 100, n)
        out.append((f"ties_n{n}", x))
        y = x.copy()
        y[n * 2 // 3] = -100
        y[n // 3] = 200
        out.append((f"planted_n{n}", y))
    return out


def make(exe: str) -> dict:
    d = Driver(exe)
    rng = np.random.default_rng(20250901)
    fx: dict[str, np.ndarray] = {"omp_threads": np.array(OMP_THREADS)}

    # ---- reducers (seq for every type; omp for the integer types: their
    # sums, extremes and bit ops do not depend on the combine order)
    base = reduce_inputs(rng)
    for t in ("i32", "i64", "f32", "f64"):
        ins = [(nm, x.astype(NP[t])) for nm, x in base]
        if t in ("f32", "f64"):
            ins.append(("uniform_n4099", rng.uniform(-1, 1, 4099).astype(NP[t])))
        for nm, x in ins:
            for pol in (("seq", "omp") if t in ("i32", "i64") else ("seq",)):
                o = d.path()
                d.run("reduce", t, pol, x.size, d.path(x), o)
                raw = np.fromfile(o, dtype=np.uint8)
                fx[f"reduce/{t}/in/{nm}"] = x
                fx[f"reduce/{t}/{pol}/{nm}/out"] = raw
            o = d.path()
            d.run("params", t, x.size, d.path(x), o)
            fx[f"params/{t}/seq/{nm}/out"] = np.fromfile(o, dtype=np.uint8)

    # ---- scans: iota (RAJA's scan tests) and random data, every kind and op
    for t in ("i32", "i64", "f32", "f64"):
        ins = [("iota_n357", np.arange(357).astype(NP[t])),
               ("empty", np.zeros(0, NP[t])), ("one", np.array([7], NP[t]))]
        if t in ("i32", "i64"):
            ins.append(("rand_n2000", rng.integers(-1000, 1000, 2000).astype(NP[t])))
        else:
            ins.append(("rand_n2000", rng.uniform(-1, 1, 2000).astype(NP[t])))
        ops = ("plus", "minimum", "maximum") if t in ("i32", "i64") else ("plus",)
        for nm, x in ins:
            for pol in ("seq", "omp"):
                for kind in ("inclusive", "exclusive", "inclusive_inplace", "exclusive_inplace"):
                    for op in ops:
                        inits = [None]
                        if kind.startswith("exclusive") and op == "plus":
                            inits.append(13)
                        for init in inits:
                            o = d.path()
                            args = ["scan", t, pol, kind, op, x.size, d.path(x), o]
                            if init is not None:
                                args.append(init)
                            d.run(*args)
                            key = f"scan/{t}/{pol}/{kind}/{op}/{'init13' if init is not None else 'noinit'}/{nm}"
                            fx[f"scan/{t}/in/{nm}"] = x
                            fx[key + "/out"] = np.fromfile(o, dtype=NP[t])
    for pol in ("seq", "omp"):      # a long iota scan, as in RAJA's tests
        x = np.arange(32000).astype(np.int64)
        for kind in ("inclusive", "exclusive"):
            o = d.path()
            d.run("scan", "i64", pol, kind, "plus", x.size, d.path(x), o)
            key = f"scan/i64/{pol}/{kind}/plus/noinit/iota_n32000"
            fx["scan/i64/in/iota_n32000"] = x
            fx[key + "/out"] = np.fromfile(o, dtype=np.int64)

    # ---- sorts: RAJA's sort-test sizes, keys uniform in [-N, N] (unsigned:
    # [0, 2N]); floats add signed zeros and duplicates
    for t in ("u32", "i32", "u64", "i64", "f32", "f64"):
        for n in (0, 1, 10, 100, 1000):
            if t.startswith("u"):
                k = rng.integers(0, 2 * n + 1, n).astype(NP[t])
            elif t.startswith("i"):
                k = rng.integers(-n, n + 1, n).astype(NP[t])
            else:
                k = rng.integers(-n, n + 1, n).astype(NP[t]) / NP[t](4)
                if n >= 10:
                    k[1] = NP[t](0.0)
                    k[2] = -NP[t](0.0)
                    k[n // 2] = k[n // 3]
            v = np.arange(n, dtype=np.int32)
            for pol in ("seq", "omp"):
                for kind in ("sort", "stable_sort"):
                    for dr in ("asc", "desc"):
                        key = f"sort/{t}/{pol}/{kind}/{dr}/n{n}"
                        ko = d.path()
                        d.run("sort", t, pol, kind, dr, n, d.path(k), ko)
                        fx[f"sort/{t}/in/n{n}"] = k
                        fx[key + "/out"] = np.fromfile(ko, dtype=NP[t])
                        ko, vo = d.path(), d.path()
                        d.run("sort", t, pol, kind, dr, n, d.path(k), ko, d.path(v), vo)
                        fx[key + "/pairs_out"] = np.fromfile(ko, dtype=NP[t])
                        fx[key + "/pairs_vout"] = np.fromfile(vo, dtype=np.int32)

    # ---- MultiReduceSum histogram of Zipf(1.1) bins
    for nb in (256, 65536):
        w = 1.0 / np.arange(1, nb + 1) ** 1.1
        cdf = np.cumsum(w) / w.sum()
        b = np.searchsorted(cdf, rng.random(1 << 15), side="right").clip(0, nb - 1).astype(np.int32)
        for pol in ("seq", "omp"):
            o = d.path()
            d.run("hist", pol, b.size, nb, d.path(b), o)
            fx[f"hist/in/bins{nb}"] = b
            fx[f"hist/{pol}/bins{nb}/out"] = np.fromfile(o, dtype=np.int64)

    # ---- forall daxpy y += 2.5 x
    x, y = rng.uniform(-1, 1, 4099), rng.uniform(-1, 1, 4099)
    for pol in ("seq", "omp"):
        o = d.path()
        d.run("daxpy", pol, x.size, "2.5", d.path(x), d.path(y), o)
        fx["daxpy/x"], fx["daxpy/y"] = x, y
        fx[f"daxpy/{pol}/out"] = np.fromfile(o, dtype=np.float64)

    # ---- WorkGroup (seq_work, ordered), run twice
    nl, total = 64, 8192
    b = rng.integers(0, total, nl).astype(np.int64)
    e = np.minimum(b + rng.integers(0, 600, nl), total).astype(np.int64)
    o = d.path()
    d.run("workgroup", nl, total, d.path(b), d.path(e), o)
    fx["workgroup/begins"], fx["workgroup/ends"] = b, e
    fx["workgroup/out"] = np.fromfile(o, dtype=np.int64)
    return fx


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    a = ap.parse_args()
    from oracle.refbuild.build_ref import build_ref
    exe = build_ref(a.ref)
    fx = make(exe)
    np.savez_compressed(OUT, **fx)
    print(f"{OUT}: {len(fx)} arrays, {os.path.getsize(OUT) / 1e6:.2f} MB")


if __name__ == "__main__":
    main()
