"""The allocation-free FP64 sum against the arena-backed entry point.

b200_reduce_sum_f64_noalloc exists for callers that cannot let a library
allocate device memory: hosts whose memory manager owns all of the GPU's
memory, and latency-critical loops that cannot afford allocator calls.  It
must give the same sums as b200_reduce_sum_f64, including on back-to-back
calls that reuse its static scratch.  This file is collected last so that a
run stopping at the first failure has already run every other test; it also
passes on its own in a fresh process.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sum(lib, name, x, mode, out):
    import torch
    rc = getattr(lib, name)(x.data_ptr(), x.numel(), mode, out.data_ptr(),
                            torch.cuda.current_stream().cuda_stream)
    assert rc == 0, lib.b200_last_error_string()


def test_noalloc_sum_matches_arena_sum_twice_in_a_row(prims):
    """Both entry points run the same kernel, grid and chunk mapping, so the
    sums must agree bit for bit in every mode, on aligned inputs (16-byte
    vector loads) and on a view one element in (scalar loads)."""
    import torch
    from raja_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(42)
    for n in (0, 1, 4097, (1 << 20) + 3, 1 << 24):
        base = torch.from_numpy(rng.uniform(-1, 1, n + 1)).cuda()
        for x in (base[:n], base[1:]):
            for mode in (0, 1, 2, 3):
                ref = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
                _sum(lib, "b200_reduce_sum_f64", x, mode, ref)
                for _ in range(2):  # two calls in a row share the static scratch
                    got = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
                    _sum(lib, "b200_reduce_sum_f64_noalloc", x, mode, got)
                    torch.cuda.synchronize()
                    g, r = got.cpu().view(torch.int64).item(), ref.cpu().view(torch.int64).item()
                    assert g == r, (n, mode, x.data_ptr() % 16, got.item(), ref.item())
    prims.synchronize()


def test_noalloc_rejects_deterministic_sizes_beyond_its_scratch(prims):
    import torch
    from raja_gb300 import _lib
    lib = _lib.load()
    n = (1 << 24) + 1
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = lib.b200_reduce_sum_f64_noalloc(x.data_ptr(), n, 2, out.data_ptr(),
                                         torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.B200_ERR_ARG
    assert b"maximum" in lib.b200_last_error_string()
    # the non-deterministic modes take the same n
    rc = lib.b200_reduce_sum_f64_noalloc(x.data_ptr(), n, 0, out.data_ptr(),
                                         torch.cuda.current_stream().cuda_stream)
    assert rc == 0
    prims.synchronize()
    assert out.item() == 0.0
