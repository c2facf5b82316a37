"""ctypes binding of libb200prims.so (the C ABI declared in include/b200prims.h).

The library is loaded from this package directory.  There is no fallback:
if the shared object is missing or fails to load, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libb200prims.so")

B200_OK = 0
B200_ERR_ARG = 1
B200_ERR_CUDA = 2
B200_ERR_TIMEOUT = 3
B200_ERR_NOMEM = 4
B200_ERR_UNSUPPORTED = 5

MODE_NAIVE = 0
MODE_COMPENSATED = 1
MODE_DETERMINISTIC = 2

OP_SUM = 0
OP_MIN = 1
OP_MAX = 2

_P = C.c_void_p
_SZ = C.c_size_t
_I = C.c_int

# ctypes scalar type per dtype suffix
SCALAR = {
    "f32": C.c_float, "f64": C.c_double, "i32": C.c_int32, "i64": C.c_int64,
    "u32": C.c_uint32, "u64": C.c_uint64,
}


def _signatures() -> dict[str, tuple]:
    """name -> (restype, argtypes) for every exported entry point."""
    sig: dict[str, tuple] = {
        "b200_abi_version": (_I, []),
        "b200_last_error_string": (C.c_char_p, []),
        "b200_stream_synchronize": (_I, [_P]),
        "b200_status_word_address": (_I, [_P]),
        "b200_set_spin_limit": (_I, [C.c_uint64]),
        "b200_selftest_scan_timeout": (_I, [_P]),
        "b200_device_info": (_I, [_P, _P, _P]),
        "b200_release_scratch": (_I, []),
        "b200_prof_enable": (_I, [_I]),
        "b200_prof_reset": (_I, []),
        "b200_prof_read": (_I, [_P, _SZ, _P, _P, _I]),
        "b200_forall_axpy_f64": (_I, [C.c_double, _P, _P, _SZ, _P]),
        "b200_forall_axpy_f32": (_I, [C.c_float, _P, _P, _SZ, _P]),
        "b200_histogram_i32": (_I, [_P, _SZ, C.c_int32, _P, _P]),
        "b200_reduce_sum_f64_noalloc": (_I, [_P, _SZ, _I, _P, _P]),
    }
    for t in ("f32", "f64", "i32", "i64", "u32", "u64"):
        sig[f"b200_reduce_sum_{t}"] = (_I, [_P, _SZ, _I, _P, _P])
        sig[f"b200_reduce_min_{t}"] = (_I, [_P, _SZ, _P, _P])
        sig[f"b200_reduce_max_{t}"] = (_I, [_P, _SZ, _P, _P])
        sig[f"b200_scan_inclusive_{t}"] = (_I, [_P, _P, _SZ, _I] + ([_I] if t[0] == "f" else []) + [_P])
        sig[f"b200_scan_exclusive_{t}"] = (_I, [_P, _P, _SZ, _I, SCALAR[t]] + ([_I] if t[0] == "f" else []) + [_P])
        sig[f"b200_sort_keys_{t}"] = (_I, [_P, _SZ, _I, _P])
    for t in ("f32", "f64"):
        sig[f"b200_dot_{t}"] = (_I, [_P, _P, _SZ, _I, _P, _P])
    for t in ("f32", "f64", "i32", "i64"):
        sig[f"b200_reduce_minloc_{t}"] = (_I, [_P, _SZ, _P, _P, _P])
        sig[f"b200_reduce_maxloc_{t}"] = (_I, [_P, _SZ, _P, _P, _P])
    for t in ("i32", "i64", "u32", "u64"):
        sig[f"b200_reduce_bitor_{t}"] = (_I, [_P, _SZ, _P, _P])
        sig[f"b200_reduce_bitand_{t}"] = (_I, [_P, _SZ, _P, _P])
    for t in ("u32", "u64", "f32"):
        sig[f"b200_sort_keys_copy_{t}"] = (_I, [_P, _P, _SZ, _I, _P])
    for kv in ("u32_i32", "u32_u32", "i32_i32", "f32_i32", "u64_i32", "u64_i64", "i64_i64",
               "f64_i64", "f64_i32", "i64_i32", "u32_i64", "i32_i64", "f32_i64"):
        sig[f"b200_sort_pairs_{kv}"] = (_I, [_P, _P, _SZ, _I, _P])
    for kv in ("f32_i32", "u32_i32"):
        sig[f"b200_sort_pairs_copy_{kv}"] = (_I, [_P, _P, _P, _P, _SZ, _I, _P])
    for t in ("i32", "i64", "u32", "u64", "f32", "f64"):
        for op in ("sum", "min", "max") + (("bitor", "bitand") if t[0] != "f" else ()):
            sig[f"b200_multi_reduce_{op}_{t}"] = (_I, [_P, _P, _SZ, C.c_int32, _P, _P])
    sig.update({
        "b200_batch_plan_create": (_I, [_P, _I, _P]),
        "b200_batch_plan_destroy": (_I, [_P]),
        "b200_batch_plan_info": (_I, [_P, _P, _P, _P, _P]),
        "b200_batch_plan_offsets": (_P, [_P]),
        "b200_batch_plan_set_shape": (_I, [_P, _I, _I]),
        "b200_batched_axpy_sum_f32": (_I, [_P, C.c_float, _P, _P, _P, _I, _P]),
        "b200_batch_autotune_axpy_sum_f32": (_I, [_P, C.c_float, _P, _P, _P, _I, _P]),
        "b200_loop_axpy_sum_f32": (_I, [C.c_float, _P, _P, _SZ, _P, _I, _P]),
        "b200_loops_axpy_sum_f32": (_I, [_I, _P, C.c_float, _P, _P, _P, _I, _P]),
        "b200_segmented_scan_inclusive_i32": (_I, [_P, _P, _P, _P]),
        "b200_segmented_scan_exclusive_i32": (_I, [_P, _P, _P, _P]),
        "b200_segmented_sort_keys_u32": (_I, [_P, _P, _I, _P]),
        "b200_jacobi_plan_create": (_I, [_P, _P, _P, _I, _P]),
        "b200_jacobi_plan_destroy": (_I, [_P]),
        "b200_jacobi_plan_info": (_I, [_P, _P, _P, _P]),
        "b200_jacobi_plan_offsets": (_P, [_P]),
        "b200_jacobi_sweep_f64": (_I, [_P, _P, _P, _P, _P, _P]),
        "b200_jacobi_mesh_sweep_f64": (_I, [_I, _I, _I, _P, _P, _P, _P, _P]),
        "b200_graph_capture_begin": (_I, [_P]),
        "b200_graph_capture_end": (_I, [_P, _P]),
        "b200_graph_launch": (_I, [_P, _P]),
        "b200_graph_destroy": (_I, [_P]),
    })
    return sig


SIGNATURES = _signatures()

_lock = threading.Lock()
_lib: C.CDLL | None = None


def load(path: str | None = None) -> C.CDLL:
    """Load libb200prims.so and attach argument types (raises if absent)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise RuntimeError(
                f"libb200prims.so not found at {p}: build it with "
                "`python -m raja_gb300.build` (or __graft_entry__.build()); "
                "there is no CPU fallback")
        lib = C.CDLL(p)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


class B200Error(RuntimeError):
    """A libb200prims call returned a non-zero status."""

    def __init__(self, name: str, code: int, msg: str):
        super().__init__(f"{name} failed with status {code}: {msg}")
        self.code = code


def check(name: str, rc: int) -> None:
    if rc != B200_OK:
        msg = load().b200_last_error_string()
        raise B200Error(name, rc, msg.decode() if msg else "")


def call(name: str, *args) -> None:
    lib = load()
    check(name, getattr(lib, name)(*args))
