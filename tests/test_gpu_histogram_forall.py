"""Histogram (MultiReduceSum +1) and the daxpy forall body through the
C ABI vs the oracle and golden fixtures."""
import os

import numpy as np
import pytest

from conftest import to_dev, to_host

pytestmark = pytest.mark.gpu

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_golden_histogram(prims):
    g = np.load(os.path.join(G, "histogram.npz"))
    np.testing.assert_array_equal(to_host(prims.histogram(to_dev(g["z256"]), 256)), g["h256"])
    np.testing.assert_array_equal(to_host(prims.histogram(to_dev(g["z64k"]), 65536)), g["h64k"])


@pytest.mark.parametrize("nbins", [1, 7, 256, 2048, 2049, 65536, 100000])
def test_histogram_bit_exact(prims, orc, nbins):
    import sys
    sys.path.insert(0, G)
    from make_golden import zipf_bins
    rng = np.random.default_rng(nbins)
    for n in (0, 1, 33, 4097, 1000003):
        x = zipf_bins(rng, n, nbins)
        if n > 10:
            x[3], x[4], x[5] = -1, nbins, 2 ** 31 - 1       # not counted
        exp = orc.histogram(x, nbins).astype(np.int64)
        np.testing.assert_array_equal(to_host(prims.histogram(to_dev(x), nbins)), exp)
        if n > 3:   # misaligned start
            np.testing.assert_array_equal(to_host(prims.histogram(to_dev(x)[1:], nbins)),
                                          orc.histogram(x[1:], nbins).astype(np.int64))


@pytest.mark.parametrize("nbins", [65536, 70001, 114000])
def test_histogram_hot_bins_many_bins(prims, orc, nbins):
    """More bins than fit in shared memory as 32-bit counts (the rest are
    counted in global memory): two adjacent hot bins take ~100k hits per
    block, the last bin and scattered others a few."""
    import torch
    n = 1 << 24
    g = torch.Generator(device="cuda")
    g.manual_seed(nbins)
    x = torch.randint(0, nbins, (n,), generator=g, device="cuda", dtype=torch.int32)
    hot = torch.rand(n, generator=g, device="cuda") < 0.9
    x = torch.where(hot, torch.where(torch.arange(n, device="cuda") % 3 == 0, 41, 40), x).to(torch.int32)
    x[::1000] = nbins - 1
    xh = x.cpu().numpy()
    exp = orc.histogram(xh, nbins).astype(np.int64)
    assert exp[40] > 1 << 22 and exp[41] > 1 << 21
    np.testing.assert_array_equal(to_host(prims.histogram(x, nbins)), exp)


def test_histogram_accumulates(prims):
    import torch
    x = torch.randint(0, 16, (100000,), dtype=torch.int32, device="cuda")
    c = prims.histogram(x, 16)
    prims.histogram(x, 16, counts=c)
    assert torch.equal(c, 2 * torch.bincount(x.long(), minlength=16))


def test_golden_axpy(prims):
    g = np.load(os.path.join(G, "axpy.npz"))
    y = to_dev(g["y"])
    prims.forall_axpy(float(g["a"]), to_dev(g["x"]), y)
    # fused multiply-add on the GPU vs two roundings: within 1 ulp
    np.testing.assert_allclose(to_host(y), g["y_out"], rtol=2 ** -52, atol=2 ** -53)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_axpy_vs_oracle(prims, orc, dt):
    u = 2.0 ** -23 if dt == np.float32 else 2.0 ** -52
    for n in (0, 1, 5, 4096, 4099, (1 << 20) + 3):
        rng = np.random.default_rng(n)
        x = rng.uniform(-1, 1, n).astype(dt)
        y = rng.uniform(-1, 1, n).astype(dt)
        dy = to_dev(y)
        prims.forall_axpy(2.5, to_dev(x), dy)
        exp = orc.axpy(2.5, x, y.copy())
        bound = u * (np.abs(exp) + 2.5 * np.abs(x))
        assert np.all(np.abs(to_host(dy) - exp) <= bound)
        if n > 4:
            dy = to_dev(y)
            prims.forall_axpy(2.5, to_dev(x)[1:], dy[1:])   # misaligned
            exp = orc.axpy(2.5, x[1:], y[1:].copy())
            assert np.all(np.abs(to_host(dy)[1:] - exp) <= u * (np.abs(exp) + 2.5 * np.abs(x[1:])))
