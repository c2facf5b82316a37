"""ORACLE -- test infrastructure only (see oracle/oracle.cpp).

numpy-facing ctypes wrappers over liboracle.so, the CPU restatement of
RAJA's seq_exec / omp_parallel_for_exec semantics for the primitive path,
pinned bit for bit against outputs of RAJA's own host policies
(tests/golden/ref_fixtures.npz, tests/test_ref_fixtures.py).
Only tests/, __graft_entry__.smoke() and the CPU-baseline legs of bench.py
use it, always as the checker or the timed CPU reference, never as the
product.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .build_oracle import OUT as LIB_PATH, build

_lib = None

_CT = {np.dtype(np.float32): C.c_float, np.dtype(np.float64): C.c_double,
       np.dtype(np.int32): C.c_int32, np.dtype(np.int64): C.c_int64,
       np.dtype(np.uint32): C.c_uint32, np.dtype(np.uint64): C.c_uint64}
_SFX = {np.dtype(np.float32): "f32", np.dtype(np.float64): "f64",
        np.dtype(np.int32): "i32", np.dtype(np.int64): "i64",
        np.dtype(np.uint32): "u32", np.dtype(np.uint64): "u64"}
OPS = {"plus": 0, "sum": 0, "minimum": 1, "min": 1, "maximum": 2, "max": 2}


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = C.CDLL(LIB_PATH)
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _fn(name, res, args):
    f = getattr(lib(), name)
    f.restype = res
    f.argtypes = args
    return f


def max_threads() -> int:
    return _fn("orc_max_threads", C.c_int, [])()


def set_threads(n: int) -> None:
    _fn("orc_set_threads", None, [C.c_int])(int(n))


# ---------------------------------------------------------------- forall
def axpy(a: float, x: np.ndarray, y: np.ndarray, parallel: bool = False) -> np.ndarray:
    """y += a*x in place (seq or omp loop); returns y."""
    sfx = _SFX[x.dtype]
    f = _fn(f"orc_{'omp' if parallel else 'seq'}_axpy_{sfx}", None,
            [_CT[x.dtype], C.c_void_p, C.c_void_p, C.c_int64])
    f(a, _p(x), _p(y), x.size)
    return y


# -------------------------------------------------------------- reducers
def reduce_sum(x: np.ndarray, init=0, parallel: bool = False):
    x = np.ascontiguousarray(x)
    sfx = _SFX[x.dtype]
    ct = _CT[x.dtype]
    if parallel:
        if sfx not in ("f32", "f64"):
            raise TypeError("omp sum restated for f32/f64")
        f = _fn(f"orc_omp_sum_{sfx}", ct, [C.c_void_p, C.c_int64, ct])
    else:
        f = _fn(f"orc_seq_sum_{sfx}", ct, [C.c_void_p, C.c_int64, ct])
    return f(_p(x), x.size, ct(init))


def dot(x: np.ndarray, y: np.ndarray, init=0.0, parallel: bool = False):
    sfx = _SFX[x.dtype]
    ct = _CT[x.dtype]
    f = _fn(f"orc_{'omp' if parallel else 'seq'}_dot_{sfx}", ct,
            [C.c_void_p, C.c_void_p, C.c_int64, ct])
    return f(_p(x), _p(y), x.size, ct(init))


def _limits(dt):
    if dt.kind == "f":
        fi = np.finfo(dt)
        return fi.max, -fi.max
    ii = np.iinfo(dt)
    return ii.max, ii.min


def reduce_minloc(x: np.ndarray, init_val=None, init_loc: int = -1, parallel: bool = False):
    x = np.ascontiguousarray(x)
    sfx, ct = _SFX[x.dtype], _CT[x.dtype]
    val, loc = ct(), C.c_int64()
    if parallel:
        _fn(f"orc_omp_minloc_{sfx}", None, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p])(
            _p(x), x.size, C.byref(val), C.byref(loc))
    else:
        iv = _limits(x.dtype)[0] if init_val is None else init_val
        _fn(f"orc_seq_minloc_{sfx}", None,
            [C.c_void_p, C.c_int64, ct, C.c_int64, C.c_void_p, C.c_void_p])(
            _p(x), x.size, ct(iv), init_loc, C.byref(val), C.byref(loc))
    return val.value, loc.value


def reduce_maxloc(x: np.ndarray, init_val=None, init_loc: int = -1, parallel: bool = False):
    x = np.ascontiguousarray(x)
    sfx, ct = _SFX[x.dtype], _CT[x.dtype]
    val, loc = ct(), C.c_int64()
    if parallel:
        _fn(f"orc_omp_maxloc_{sfx}", None, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p])(
            _p(x), x.size, C.byref(val), C.byref(loc))
    else:
        iv = _limits(x.dtype)[1] if init_val is None else init_val
        _fn(f"orc_seq_maxloc_{sfx}", None,
            [C.c_void_p, C.c_int64, ct, C.c_int64, C.c_void_p, C.c_void_p])(
            _p(x), x.size, ct(iv), init_loc, C.byref(val), C.byref(loc))
    return val.value, loc.value


def reduce_min(x: np.ndarray, init=None):
    x = np.ascontiguousarray(x)
    sfx, ct = _SFX[x.dtype], _CT[x.dtype]
    iv = _limits(x.dtype)[0] if init is None else init
    return _fn(f"orc_seq_min_{sfx}", ct, [C.c_void_p, C.c_int64, ct])(_p(x), x.size, ct(iv))


def reduce_max(x: np.ndarray, init=None):
    x = np.ascontiguousarray(x)
    sfx, ct = _SFX[x.dtype], _CT[x.dtype]
    iv = _limits(x.dtype)[1] if init is None else init
    return _fn(f"orc_seq_max_{sfx}", ct, [C.c_void_p, C.c_int64, ct])(_p(x), x.size, ct(iv))


def reduce_bitor(x: np.ndarray, init=0):
    x = np.ascontiguousarray(x)
    sfx, ct = _SFX[x.dtype], _CT[x.dtype]
    return _fn(f"orc_seq_bitor_{sfx}", ct, [C.c_void_p, C.c_int64, ct])(_p(x), x.size, ct(init))


def reduce_bitand(x: np.ndarray, init=-1):
    x = np.ascontiguousarray(x)
    sfx, ct = _SFX[x.dtype], _CT[x.dtype]
    if x.dtype.kind == "u" and init == -1:
        init = np.iinfo(x.dtype).max
    return _fn(f"orc_seq_bitand_{sfx}", ct, [C.c_void_p, C.c_int64, ct])(_p(x), x.size, ct(init))


# ------------------------------------------------------------------ scans
def scan(x: np.ndarray, op="plus", exclusive: bool = False, init=None, parallel: bool = False,
         out: np.ndarray | None = None) -> np.ndarray:
    x = np.ascontiguousarray(x)
    sfx, ct = _SFX[x.dtype], _CT[x.dtype]
    o = OPS[op] if isinstance(op, str) else int(op)
    if init is None:
        hi, lo = _limits(x.dtype)
        init = {0: 0, 1: hi, 2: lo}[o]
    if out is None:
        out = np.empty_like(x)
    f = _fn(f"orc_scan_{sfx}", C.c_int,
            [C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_int, ct, C.c_int])
    rc = f(_p(x), _p(out), x.size, o, int(exclusive), ct(init), int(parallel))
    if rc:
        raise ValueError(f"oracle scan failed ({rc})")
    return out


# ------------------------------------------------------------------ sorts
def sort(keys: np.ndarray, descending: bool = False, parallel: bool = False,
         stable: bool = True) -> np.ndarray:
    """Sorted copy of keys."""
    k = np.array(keys, copy=True)
    sfx = _SFX[k.dtype]
    _fn(f"orc_sort_{sfx}", None, [C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_int])(
        _p(k), k.size, int(descending), int(parallel), int(stable))
    return k


def sort_inplace(k: np.ndarray, descending: bool = False, parallel: bool = False,
                 stable: bool = True) -> np.ndarray:
    """Sort a contiguous array in place (RAJA's sorts are in place)."""
    assert k.flags.c_contiguous
    _fn(f"orc_sort_{_SFX[k.dtype]}", None, [C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_int])(
        _p(k), k.size, int(descending), int(parallel), int(stable))
    return k


def sort_pairs_inplace(k: np.ndarray, v: np.ndarray, descending: bool = False,
                       parallel: bool = False, stable: bool = True):
    assert k.flags.c_contiguous and v.flags.c_contiguous and k.size == v.size
    name = f"orc_sort_pairs_{_SFX[k.dtype]}_{_SFX[v.dtype]}"
    _fn(name, None, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_int])(
        _p(k), _p(v), k.size, int(descending), int(parallel), int(stable))
    return k, v


def sort_pairs(keys: np.ndarray, vals: np.ndarray, descending: bool = False,
               parallel: bool = False, stable: bool = True):
    k = np.array(keys, copy=True)
    v = np.array(vals, copy=True)
    name = f"orc_sort_pairs_{_SFX[k.dtype]}_{_SFX[v.dtype]}"
    _fn(name, None, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_int])(
        _p(k), _p(v), k.size, int(descending), int(parallel), int(stable))
    return k, v


# -------------------------------------------------------------- histogram
def histogram(x: np.ndarray, nbins: int, parallel: bool = False) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.int32)
    counts = np.zeros(nbins, dtype=np.uint64)
    _fn(f"orc_{'omp' if parallel else 'seq'}_histogram_i32", None,
        [C.c_void_p, C.c_int64, C.c_int32, C.c_void_p])(_p(x), x.size, nbins, _p(counts))
    return counts


def multi_reduce(op: str, bins: np.ndarray, vals: np.ndarray, out: np.ndarray) -> np.ndarray:
    """MultiReduce{Sum,Min,Max,BitOr,BitAnd}: out[b] combined in place with
    every vals[i] whose bins[i] == b, in index order (seq rule)."""
    bins = np.ascontiguousarray(bins, dtype=np.int32)
    vals = np.ascontiguousarray(vals)
    assert out.dtype == vals.dtype and out.flags.c_contiguous
    _fn(f"orc_multi_reduce_{op}_{_SFX[vals.dtype]}", None,
        [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p])(
        _p(bins), _p(vals), vals.size, out.size, _p(out))
    return out


# ------------------------------------------------------ exact arithmetic
def exact_sum(x: np.ndarray) -> tuple[float, float]:
    """Exact sum as (hi, lo): hi = round(sum), lo = round(sum - hi)."""
    x = np.ascontiguousarray(x)
    hi, lo = C.c_double(), C.c_double()
    _fn(f"orc_exact_sum_{_SFX[x.dtype]}", None, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p])(
        _p(x), x.size, C.byref(hi), C.byref(lo))
    return hi.value, lo.value


def exact_dot(x: np.ndarray, y: np.ndarray) -> tuple[float, float]:
    hi, lo = C.c_double(), C.c_double()
    _fn(f"orc_exact_dot_{_SFX[x.dtype]}", None,
        [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p])(
        _p(x), _p(y), x.size, C.byref(hi), C.byref(lo))
    return hi.value, lo.value


def exact_abs_sum_f32(x: np.ndarray) -> float:
    return _fn("orc_exact_abs_sum_f32", C.c_double, [C.c_void_p, C.c_int64])(_p(x), x.size)


def dd_scan_f32(x: np.ndarray) -> np.ndarray:
    """Inclusive prefix sums of f32 data carried in double-double."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    out = np.empty(x.size, dtype=np.float64)
    _fn("orc_dd_scan_f32", None, [C.c_void_p, C.c_int64, C.c_void_p])(_p(x), x.size, _p(out))
    return out


# ------------------------------------------------------------------ jacobi
def jacobi_sweep(u: np.ndarray, unew: np.ndarray, f: np.ndarray | None, shape) -> float:
    """One 7-point sweep of one mesh (shape = (nx, ny, nz), x fastest);
    writes unew's interior and returns the max residual."""
    nx, ny, nz = shape
    fp = _p(f) if f is not None else None
    fn = _fn("orc_jacobi_sweep_f64", C.c_double,
             [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p])
    return fn(nx, ny, nz, _p(u), _p(unew), fp)
