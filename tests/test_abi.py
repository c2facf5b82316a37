"""The C ABI library loads and exports every symbol include/b200prims.h
declares; host-side argument validation (no device work) behaves."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "b200prims.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:int|const char\*|const int64_t\*)\s+(b200_\w+)\s*\(", src, flags=re.M)
    assert len(names) > 60
    return names


@pytest.fixture(scope="module")
def lib():
    from raja_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        import raja_gb300.build
        raja_gb300.build.build()
    return _lib.load()


def test_every_declared_symbol_is_exported_and_bound(lib):
    from raja_gb300 import _lib
    names = declared_functions()
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    unbound = [n for n in names if n not in _lib.SIGNATURES]
    assert not unbound, unbound
    extra = [n for n in _lib.SIGNATURES if n not in names]
    assert not extra, extra


def test_abi_version_and_error_string(lib):
    assert lib.b200_abi_version() == 1
    assert isinstance(lib.b200_last_error_string(), bytes)


def test_argument_validation_without_device_work(lib):
    from raja_gb300 import _lib
    # nbins <= 0 is rejected before any CUDA call
    assert lib.b200_histogram_i32(None, 10, 0, None, None) == _lib.B200_ERR_ARG
    assert b"nbins" in lib.b200_last_error_string()
    # null output of a reduction
    assert lib.b200_reduce_sum_f64(None, 10, 0, None, None) == _lib.B200_ERR_ARG
    # sorts cap n below 2^32
    assert lib.b200_sort_keys_u32(C.c_void_p(16), 1 << 32, 0, None) == _lib.B200_ERR_ARG
    # null input pointers with n > 0
    assert lib.b200_scan_inclusive_i32(None, None, 5, 0, None) == _lib.B200_ERR_ARG
    # partially overlapping scan buffers
    base = 1 << 20
    assert lib.b200_scan_inclusive_i32(C.c_void_p(base), C.c_void_p(base + 8), 100, 0,
                                       None) == _lib.B200_ERR_ARG
    # unknown reduction mode
    assert lib.b200_reduce_sum_f32(C.c_void_p(base), 10, 7, C.c_void_p(base), None) == _lib.B200_ERR_ARG
    # empty scans and histograms are no-ops
    assert lib.b200_scan_exclusive_i64(None, None, 0, 0, 0, None) == _lib.B200_OK
    assert lib.b200_histogram_i32(None, 0, 16, C.c_void_p(base), None) == _lib.B200_OK


def test_python_mirror_raises_loudly_without_library(tmp_path):
    from raja_gb300 import _lib
    saved = _lib._lib
    try:
        _lib._lib = None
        with pytest.raises(RuntimeError, match="no CPU fallback"):
            _lib.load(str(tmp_path / "missing.so"))
    finally:
        _lib._lib = saved
