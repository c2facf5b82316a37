"""Failure paths without a GPU fault: the bounded look-back wait gives up
with a status the host reads, and the context stays usable."""
import pytest

pytestmark = pytest.mark.gpu


def test_lookback_timeout_is_reported_and_context_survives(prims):
    import torch
    from raja_gb300 import _lib
    prims.synchronize()
    prims.set_spin_limit(2000)
    try:
        _lib.call("b200_selftest_scan_timeout", torch.cuda.current_stream().cuda_stream)
        with pytest.raises(prims.B200Error) as ei:
            prims.synchronize()
        assert ei.value.code == _lib.B200_ERR_TIMEOUT
        assert "scan" in str(ei.value)
    finally:
        prims.set_spin_limit(0)
    # the status was cleared and the device still works
    prims.synchronize()
    x = torch.arange(1, 100001, dtype=torch.int64, device="cuda")
    assert prims.reduce_sum(x) == 100000 * 100001 // 2
    out = prims.inclusive_scan(x)
    assert out[-1].item() == 100000 * 100001 // 2


def test_bad_arguments_raise(prims):
    import torch
    x = torch.zeros(10, dtype=torch.int32, device="cuda")
    with pytest.raises(prims.B200Error):
        prims.histogram(x, 0)
    with pytest.raises(prims.B200Error):
        prims.inclusive_scan(x, op=9)


def test_status_word_is_host_readable_after_the_stream_syncs(prims):
    """The status word sits in mapped host memory: after the stream has
    synchronised, the host reads the timeout bit directly; the next
    b200_stream_synchronize() reports and clears it."""
    import ctypes as C
    import torch
    from raja_gb300 import _lib
    lib = _lib.load()
    prims.synchronize()
    addr = C.c_void_p()
    assert lib.b200_status_word_address(C.byref(addr)) == 0 and addr.value
    word = C.cast(addr, C.POINTER(C.c_uint32))
    assert word[0] == 0
    stream = torch.cuda.current_stream()
    prims.set_spin_limit(2000)
    try:
        _lib.call("b200_selftest_scan_timeout", stream.cuda_stream)
        stream.synchronize()
        assert word[0] & 1                       # the scan look-back bit
        with pytest.raises(prims.B200Error):
            prims.synchronize()
    finally:
        prims.set_spin_limit(0)
    assert word[0] == 0
    prims.synchronize()
