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
