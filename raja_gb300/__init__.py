"""raja_gb300 -- GB300-native backend for RAJA's data-parallel primitive path.

Python host mirror of the reference interface over the C ABI of
libb200prims.so (include/b200prims.h).  Names follow RAJA's front-ends:

  forall (fixed-type bodies)   forall_axpy                      pattern/forall.hpp
  reducers                     reduce_sum / reduce_min / ...     pattern/reduce.hpp
                               dot, reduce_minloc/maxloc,
                               reduce_bitor/bitand
  scans                        inclusive_scan, exclusive_scan,  pattern/scan.hpp:49-441
                               inclusive_scan_inplace,
                               exclusive_scan_inplace
  sorts                        sort, stable_sort, sort_pairs,   pattern/sort.hpp:59-451
                               stable_sort_pairs
  MultiReduceSum (+1 body)     histogram                        pattern/multi_reduce.hpp

Tensors are torch CUDA tensors (device memory); work is enqueued on the
current torch stream.  Like RAJA's synchronous cuda_exec policies, calls wait
for completion and raise on error unless `sync=False` is passed (errors from
a bounded device wait are then reported by `synchronize()`).  There is no CPU
fallback: without the compiled library every call raises.
"""
from __future__ import annotations

import ctypes as C

from . import _lib
from ._lib import (B200Error, MODE_COMPENSATED, MODE_DETERMINISTIC, MODE_NAIVE, OP_MAX,
                   OP_MIN, OP_SUM)

__all__ = [
    "B200Error", "MODE_NAIVE", "MODE_COMPENSATED", "MODE_DETERMINISTIC",
    "load", "synchronize", "set_spin_limit", "device_info", "forall_axpy",
    "reduce_sum", "dot", "reduce_min", "reduce_max", "reduce_minloc", "reduce_maxloc",
    "reduce_bitor", "reduce_bitand", "inclusive_scan", "exclusive_scan",
    "inclusive_scan_inplace", "exclusive_scan_inplace", "sort", "stable_sort",
    "sort_pairs", "stable_sort_pairs", "sort_copy", "sort_pairs_copy", "histogram",
    "prof_enable", "prof_reset", "prof_read",
]

_OPS = {"plus": OP_SUM, "sum": OP_SUM, "minimum": OP_MIN, "min": OP_MIN,
        "maximum": OP_MAX, "max": OP_MAX}


def load():
    """Load libb200prims.so (raises RuntimeError if it is not built)."""
    return _lib.load()


def _torch():
    import torch
    return torch


def _suffix(t) -> str:
    torch = _torch()
    table = {torch.float32: "f32", torch.float64: "f64", torch.int32: "i32",
             torch.int64: "i64"}
    u32 = getattr(torch, "uint32", None)
    u64 = getattr(torch, "uint64", None)
    if u32 is not None:
        table[u32] = "u32"
    if u64 is not None:
        table[u64] = "u64"
    if t.dtype not in table:
        raise TypeError(f"unsupported dtype {t.dtype}")
    return table[t.dtype]


def _check_dev(*ts):
    for t in ts:
        if not t.is_cuda:
            raise ValueError("raja_gb300 primitives take CUDA tensors (device memory)")
        if not t.is_contiguous():
            raise ValueError("raja_gb300 primitives take contiguous tensors")


def _stream(stream=None) -> int:
    if stream is not None:
        return int(getattr(stream, "cuda_stream", stream))
    return _torch().cuda.current_stream().cuda_stream


def synchronize(stream=None) -> None:
    """Wait for the stream and raise if a bounded device wait gave up."""
    _lib.call("b200_stream_synchronize", _stream(stream))


def set_spin_limit(limit: int) -> None:
    """Test hook: bound on device polling iterations (0 = default)."""
    _lib.call("b200_set_spin_limit", int(limit))


def device_info() -> tuple[int, int, int]:
    sms, ma, mi = C.c_int(), C.c_int(), C.c_int()
    _lib.call("b200_device_info", C.byref(sms), C.byref(ma), C.byref(mi))
    return sms.value, ma.value, mi.value


def _item(t):
    """Python scalar of a 1-element device tensor (unsigned via a signed view)."""
    torch = _torch()
    name = str(t.dtype).replace("torch.", "")
    if name == "uint32":
        return int(t.view(torch.int32).item()) & 0xFFFFFFFF
    if name == "uint64":
        return int(t.view(torch.int64).item()) & 0xFFFFFFFFFFFFFFFF
    return t.item()


def _finish(sync: bool, stream) -> None:
    if sync:
        synchronize(stream)


# ------------------------------------------------------------------ forall
def forall_axpy(a: float, x, y, *, sync: bool = True, stream=None) -> None:
    """y[i] += a * x[i] over the whole range (daxpy / saxpy body)."""
    _check_dev(x, y)
    sfx = _suffix(x)
    if sfx not in ("f32", "f64") or y.dtype != x.dtype or y.numel() != x.numel():
        raise TypeError("forall_axpy takes two f32 or two f64 tensors of equal length")
    _lib.call(f"b200_forall_axpy_{sfx}", float(a), x.data_ptr(), y.data_ptr(), x.numel(),
              _stream(stream))
    _finish(sync, stream)


# ---------------------------------------------------------------- reducers
def _scalar_out(dtype):
    torch = _torch()
    return torch.empty(1, dtype=dtype, device="cuda")


def reduce_sum(x, init=0, *, mode: int = MODE_NAIVE, out=None, sync: bool = True, stream=None):
    """ReduceSum over x (plus `init`, folded on the host like RAJA's get()).

    FP inputs accumulate into a float64 result; integers wrap around in
    their own width.  With out= (a 1-element device tensor) nothing is
    synchronised and the device result is left in `out`.
    """
    torch = _torch()
    _check_dev(x)
    sfx = _suffix(x)
    acc_dtype = torch.float64 if sfx[0] == "f" else x.dtype
    res = out if out is not None else _scalar_out(acc_dtype)
    _lib.call(f"b200_reduce_sum_{sfx}", x.data_ptr(), x.numel(), int(mode), res.data_ptr(),
              _stream(stream))
    if out is not None:
        return out
    _finish(True, stream)
    v = _item(res)
    if sfx[0] == "f":
        return float(init) + v if sfx == "f64" else float(init) + v
    bits = 32 if sfx in ("i32", "u32") else 64
    r = (int(init) + int(v)) % (1 << bits)
    if sfx[0] == "i" and r >= (1 << (bits - 1)):
        r -= 1 << bits
    return r


def dot(x, y, *, mode: int = MODE_NAIVE, out=None, stream=None):
    """sum_i x[i]*y[i] (ReduceSum of products), result in float64."""
    torch = _torch()
    _check_dev(x, y)
    sfx = _suffix(x)
    if sfx not in ("f32", "f64") or y.dtype != x.dtype or y.numel() != x.numel():
        raise TypeError("dot takes two f32 or two f64 tensors of equal length")
    res = out if out is not None else _scalar_out(torch.float64)
    _lib.call(f"b200_dot_{sfx}", x.data_ptr(), y.data_ptr(), x.numel(), int(mode),
              res.data_ptr(), _stream(stream))
    if out is not None:
        return out
    _finish(True, stream)
    return res.item()


def _extremum(kind: str, x, out, stream):
    _check_dev(x)
    sfx = _suffix(x)
    res = out if out is not None else _scalar_out(x.dtype)
    _lib.call(f"b200_reduce_{kind}_{sfx}", x.data_ptr(), x.numel(), res.data_ptr(),
              _stream(stream))
    if out is not None:
        return out
    _finish(True, stream)
    return _item(res)


def reduce_min(x, *, out=None, stream=None):
    """ReduceMin (identity: the type's largest finite value)."""
    return _extremum("min", x, out, stream)


def reduce_max(x, *, out=None, stream=None):
    """ReduceMax (identity: the type's lowest finite value)."""
    return _extremum("max", x, out, stream)


def reduce_bitor(x, *, out=None, stream=None):
    return _extremum("bitor", x, out, stream)


def reduce_bitand(x, *, out=None, stream=None):
    return _extremum("bitand", x, out, stream)


def _loc(kind: str, x, out, stream):
    torch = _torch()
    _check_dev(x)
    sfx = _suffix(x)
    if out is None:
        val = _scalar_out(x.dtype)
        idx = torch.empty(1, dtype=torch.int64, device="cuda")
    else:
        val, idx = out
    _lib.call(f"b200_reduce_{kind}_{sfx}", x.data_ptr(), x.numel(), val.data_ptr(),
              idx.data_ptr(), _stream(stream))
    if out is not None:
        return out
    _finish(True, stream)
    return val.item(), int(idx.item())


def reduce_minloc(x, *, out=None, stream=None):
    """ReduceMinLoc: (value, index); ties resolve to the lowest index."""
    return _loc("minloc", x, out, stream)


def reduce_maxloc(x, *, out=None, stream=None):
    """ReduceMaxLoc: (value, index); ties resolve to the lowest index."""
    return _loc("maxloc", x, out, stream)


# ------------------------------------------------------------------- scans
def _scan(kind: str, x, out, op, init, mode, sync, stream):
    torch = _torch()
    _check_dev(x)
    sfx = _suffix(x)
    if out is None:
        out = torch.empty_like(x)
    _check_dev(out)
    if out.dtype != x.dtype or out.numel() != x.numel():
        raise TypeError("scan output must match the input's dtype and length")
    o = _OPS[op] if isinstance(op, str) else int(op)
    args = [x.data_ptr(), out.data_ptr(), x.numel(), o]
    if kind == "exclusive":
        if init is None:
            init = {OP_SUM: 0, OP_MIN: None, OP_MAX: None}[o]
            if init is None:
                if sfx[0] == "f":
                    finfo = torch.finfo(x.dtype)
                    init = finfo.max if o == OP_MIN else -finfo.max
                else:
                    info = torch.iinfo(x.dtype)
                    init = info.max if o == OP_MIN else info.min
        args.append(_lib.SCALAR[sfx](init))
    if sfx[0] == "f":
        args.append(int(mode))
    args.append(_stream(stream))
    _lib.call(f"b200_scan_{kind}_{sfx}", *args)
    _finish(sync, stream)
    return out


def inclusive_scan(x, out=None, op="plus", *, mode: int = MODE_NAIVE, sync=True, stream=None):
    """RAJA::inclusive_scan(in, out, op) -- op in plus/minimum/maximum."""
    return _scan("inclusive", x, out, op, None, mode, sync, stream)


def exclusive_scan(x, out=None, op="plus", init=None, *, mode: int = MODE_NAIVE, sync=True,
                   stream=None):
    """RAJA::exclusive_scan(in, out, op, init); init defaults to op's identity."""
    return _scan("exclusive", x, out, op, init, mode, sync, stream)


def inclusive_scan_inplace(x, op="plus", *, mode: int = MODE_NAIVE, sync=True, stream=None):
    return _scan("inclusive", x, x, op, None, mode, sync, stream)


def exclusive_scan_inplace(x, op="plus", init=None, *, mode: int = MODE_NAIVE, sync=True,
                           stream=None):
    return _scan("exclusive", x, x, op, init, mode, sync, stream)


# ------------------------------------------------------------------- sorts
def sort(keys, descending: bool = False, *, sync=True, stream=None):
    """RAJA::sort (in place).  The radix sort is stable, so it also serves
    stable_sort."""
    _check_dev(keys)
    sfx = _suffix(keys)
    _lib.call(f"b200_sort_keys_{sfx}", keys.data_ptr(), keys.numel(), int(bool(descending)),
              _stream(stream))
    _finish(sync, stream)
    return keys


stable_sort = sort


def sort_pairs(keys, vals, descending: bool = False, *, sync=True, stream=None):
    """RAJA::sort_pairs (in place, stable)."""
    _check_dev(keys, vals)
    if keys.numel() != vals.numel():
        raise ValueError("keys and values differ in length")
    name = f"b200_sort_pairs_{_suffix(keys)}_{_suffix(vals)}"
    if name not in _lib.SIGNATURES:
        raise TypeError(f"no sort_pairs for {keys.dtype} keys with {vals.dtype} values")
    _lib.call(name, keys.data_ptr(), vals.data_ptr(), keys.numel(), int(bool(descending)),
              _stream(stream))
    _finish(sync, stream)
    return keys, vals


stable_sort_pairs = sort_pairs


def sort_copy(keys_in, keys_out, descending: bool = False, *, sync=True, stream=None):
    """Out-of-place sort: keys_in is left untouched."""
    _check_dev(keys_in, keys_out)
    name = f"b200_sort_keys_copy_{_suffix(keys_in)}"
    if name not in _lib.SIGNATURES:
        raise TypeError(f"no out-of-place sort for {keys_in.dtype}")
    _lib.call(name, keys_in.data_ptr(), keys_out.data_ptr(), keys_in.numel(),
              int(bool(descending)), _stream(stream))
    _finish(sync, stream)
    return keys_out


def sort_pairs_copy(keys_in, vals_in, keys_out, vals_out, descending: bool = False, *, sync=True,
                    stream=None):
    _check_dev(keys_in, vals_in, keys_out, vals_out)
    name = f"b200_sort_pairs_copy_{_suffix(keys_in)}_{_suffix(vals_in)}"
    if name not in _lib.SIGNATURES:
        raise TypeError(f"no out-of-place sort_pairs for {keys_in.dtype}/{vals_in.dtype}")
    _lib.call(name, keys_in.data_ptr(), vals_in.data_ptr(), keys_out.data_ptr(),
              vals_out.data_ptr(), keys_in.numel(), int(bool(descending)), _stream(stream))
    _finish(sync, stream)
    return keys_out, vals_out


# --------------------------------------------------------------- histogram
def histogram(x, nbins: int, counts=None, *, sync=True, stream=None):
    """MultiReduceSum with a +1 body: counts[b] += #{i: x[i] == b}.

    Returns an int64 tensor of nbins counts (added into `counts` if given).
    """
    torch = _torch()
    _check_dev(x)
    if x.dtype != torch.int32:
        raise TypeError("histogram takes int32 bins")
    if counts is None:
        counts = torch.zeros(int(nbins), dtype=torch.int64, device=x.device)
    _lib.call("b200_histogram_i32", x.data_ptr(), x.numel(), int(nbins), counts.data_ptr(),
              _stream(stream))
    _finish(sync, stream)
    return counts


_MR_OPS = {"sum": "sum", "plus": "sum", "min": "min", "minimum": "min", "max": "max",
           "maximum": "max", "bitor": "bitor", "bit_or": "bitor", "bitand": "bitand",
           "bit_and": "bitand"}


def multi_reduce(op: str, bins, vals, nbins: int | None = None, *, out=None, init=None,
                 sync=True, stream=None):
    """RAJA::MultiReduce{Sum,Min,Max,BitOr,BitAnd}: out[b] = op(out[b], vals[i])
    for every i with bins[i] == b (bins outside [0, nbins) skipped).

    `out` (combined into) or a fresh tensor of nbins elements set to `init`
    (default: the op's identity, as MultiReduce(num_bins) starts) is returned.
    """
    torch = _torch()
    _check_dev(bins, vals)
    if bins.dtype != torch.int32:
        raise TypeError("multi_reduce takes int32 bins")
    if bins.numel() != vals.numel():
        raise ValueError("bins and vals differ in length")
    kind = _MR_OPS[op]
    sfx = _suffix(vals)
    if kind.startswith("bit") and sfx[0] == "f":
        raise TypeError("bit multi reductions take integer values")
    if out is None:
        if nbins is None:
            raise ValueError("nbins or out is required")
        bits = 8 * vals.element_size()
        if init is None:   # the op's identity
            if kind in ("sum", "bitor"):
                init = 0
            elif kind == "bitand":
                init = -1
            elif sfx[0] == "f":
                fi = torch.finfo(vals.dtype)
                init = fi.max if kind == "min" else -fi.max
            elif sfx[0] == "u":
                init = (1 << bits) - 1 if kind == "min" else 0
            else:
                info = torch.iinfo(vals.dtype)
                init = info.max if kind == "min" else info.min
        if sfx[0] == "u":   # unsigned values are held in a signed view
            init = int(init) & ((1 << bits) - 1)
            if init >= 1 << (bits - 1):
                init -= 1 << bits
            base = torch.int32 if bits == 32 else torch.int64
            out = torch.full((int(nbins),), init, dtype=base, device=vals.device).view(vals.dtype)
        else:
            out = torch.full((int(nbins),), init, dtype=vals.dtype, device=vals.device)
    elif out.dtype != vals.dtype:
        raise TypeError("out and vals differ in dtype")
    _check_dev(out)
    _lib.call(f"b200_multi_reduce_{kind}_{sfx}", bins.data_ptr(), vals.data_ptr(), vals.numel(),
              int(out.numel()), out.data_ptr(), _stream(stream))
    _finish(sync, stream)
    return out


# ----------------------------------------------------------- instrumentation
def prof_enable(on: bool = True) -> None:
    _lib.call("b200_prof_enable", int(bool(on)))


def prof_reset() -> None:
    _lib.call("b200_prof_reset")


def prof_read(cap: int = 64) -> dict[str, tuple[int, float]]:
    """{kernel name: (launches, total ms)} accumulated since prof_reset()."""
    stride = 64
    names = C.create_string_buffer(stride * cap)
    launches = (C.c_uint64 * cap)()
    ms = (C.c_double * cap)()
    k = _lib.load().b200_prof_read(names, stride, launches, ms, cap)
    out = {}
    for i in range(k):
        nm = names.raw[i * stride:(i + 1) * stride].split(b"\0", 1)[0].decode()
        out[nm] = (int(launches[i]), float(ms[i]))
    return out


# ------------------------------------------------------------- batched loops
class BatchPlan:
    """WorkPool-style plan over many loops (WorkPool::instantiate): loop i
    covers [0, lens[i]); segment i of a flattened array covers
    [offsets[i], offsets[i+1])."""

    def __init__(self, lens):
        import numpy as np
        self._lens = np.ascontiguousarray(np.asarray(lens, dtype=np.int64))
        h = C.c_void_p()
        _lib.call("b200_batch_plan_create", self._lens.ctypes.data_as(C.c_void_p),
                  int(self._lens.size), C.byref(h))
        self.handle = h.value
        self.offsets = np.concatenate([[0], np.cumsum(self._lens)]).astype(np.int64)

    @property
    def total(self) -> int:
        return int(self.offsets[-1])

    def info(self) -> dict:
        total, ntiles, tile, block = C.c_int64(), C.c_int64(), C.c_int(), C.c_int()
        _lib.call("b200_batch_plan_info", self.handle, C.byref(total), C.byref(ntiles),
                  C.byref(tile), C.byref(block))
        return {"total": total.value, "tiles": ntiles.value, "tile": tile.value,
                "block": block.value}

    def set_shape(self, block: int, items: int):
        """Pin the batched loops' launch shape (block threads x items per
        thread) to one of the autotuner's candidates."""
        _lib.call("b200_batch_plan_set_shape", self.handle, int(block), int(items))

    def close(self):
        if getattr(self, "handle", None):
            _lib.load().b200_batch_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batched_axpy_sum(plan: BatchPlan, a: float, xs, ys, sums, *, mode: int = MODE_COMPENSATED,
                     autotune: bool = False, sync=True, stream=None):
    """Every loop i: y_i += a*x_i and sums[i] = sum(y_i), in one persistent
    launch.  xs / ys: int64 CUDA tensors of device pointers; sums: float64."""
    name = "b200_batch_autotune_axpy_sum_f32" if autotune else "b200_batched_axpy_sum_f32"
    _lib.call(name, plan.handle, float(a), xs.data_ptr(), ys.data_ptr(), sums.data_ptr(),
              int(mode), _stream(stream))
    _finish(sync, stream)
    return sums


def loop_axpy_sum(a: float, x, y, out, *, mode: int = MODE_COMPENSATED, stream=None):
    """One loop's fused axpy + sum (one launch), result into out[0]."""
    _lib.call("b200_loop_axpy_sum_f32", float(a), x.data_ptr(), y.data_ptr(), x.numel(),
              out.data_ptr(), int(mode), _stream(stream))
    return out


def segmented_inclusive_scan(plan: BatchPlan, x, out=None, *, sync=True, stream=None):
    """Inclusive int32 sum scan restarting at every segment of the plan."""
    torch = _torch()
    out = torch.empty_like(x) if out is None else out
    _lib.call("b200_segmented_scan_inclusive_i32", plan.handle, x.data_ptr(), out.data_ptr(),
              _stream(stream))
    _finish(sync, stream)
    return out


def segmented_exclusive_scan(plan: BatchPlan, x, out=None, *, sync=True, stream=None):
    """Exclusive int32 sum scan restarting at every segment (0 at heads)."""
    torch = _torch()
    out = torch.empty_like(x) if out is None else out
    _lib.call("b200_segmented_scan_exclusive_i32", plan.handle, x.data_ptr(), out.data_ptr(),
              _stream(stream))
    _finish(sync, stream)
    return out


def segmented_sort(plan: BatchPlan, keys, descending: bool = False, *, sync=True, stream=None):
    """Sort each segment of a uint32 key array independently, in place."""
    _lib.call("b200_segmented_sort_keys_u32", plan.handle, keys.data_ptr(), int(bool(descending)),
              _stream(stream))
    _finish(sync, stream)
    return keys


# ------------------------------------------------------------------- jacobi
class JacobiPlan:
    """Batched 3-D meshes (x fastest, stored back to back) for Jacobi
    sweeps; shapes is a list of (nx, ny, nz)."""

    def __init__(self, shapes):
        import numpy as np
        sh = np.asarray(shapes, dtype=np.int32).reshape(-1, 3)
        self.shapes = [tuple(int(v) for v in r) for r in sh]
        nx, ny, nz = (np.ascontiguousarray(sh[:, i]) for i in range(3))
        h = C.c_void_p()
        _lib.call("b200_jacobi_plan_create", nx.ctypes.data_as(C.c_void_p),
                  ny.ctypes.data_as(C.c_void_p), nz.ctypes.data_as(C.c_void_p), len(self.shapes),
                  C.byref(h))
        self.handle = h.value
        sizes = sh[:, 0].astype(np.int64) * sh[:, 1] * sh[:, 2]
        self.offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)

    @property
    def total(self) -> int:
        return int(self.offsets[-1])

    def interior_points(self) -> int:
        return int(sum((a - 2) * (b - 2) * (c - 2) for a, b, c in self.shapes))

    def close(self):
        if getattr(self, "handle", None):
            _lib.load().b200_jacobi_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def jacobi_sweep(plan: JacobiPlan, u, unew, resid, f=None, *, sync=True, stream=None):
    """One 7-point sweep of every mesh; resid[m] = max |unew - u| (float64)."""
    _lib.call("b200_jacobi_sweep_f64", plan.handle, u.data_ptr(), unew.data_ptr(),
              f.data_ptr() if f is not None else None, resid.data_ptr(), _stream(stream))
    _finish(sync, stream)
    return resid


def jacobi_mesh_sweep(shape, u, unew, resid, f=None, *, sync=True, stream=None):
    """One sweep of one mesh (one launch)."""
    nx, ny, nz = shape
    _lib.call("b200_jacobi_mesh_sweep_f64", int(nx), int(ny), int(nz), u.data_ptr(),
              unew.data_ptr(), f.data_ptr() if f is not None else None, resid.data_ptr(),
              _stream(stream))
    _finish(sync, stream)
    return resid


# ------------------------------------------------------------------- graphs
class Graph:
    """Capture library calls issued on `stream` into a CUDA graph:

        with rg.Graph(stream) as g:
            rg.jacobi_sweep(..., sync=False, stream=stream)
        g.launch()
    """

    def __init__(self, stream):
        self.stream = _stream(stream)
        self.handle = None

    def __enter__(self):
        _lib.call("b200_graph_capture_begin", self.stream)
        return self

    def __exit__(self, *exc):
        h = C.c_void_p()
        _lib.call("b200_graph_capture_end", self.stream, C.byref(h))
        self.handle = h.value
        return False

    def launch(self):
        _lib.call("b200_graph_launch", self.handle, self.stream)

    def close(self):
        if self.handle:
            _lib.load().b200_graph_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
