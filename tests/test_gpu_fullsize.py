"""Full-size checks (N = 2^28, the bandwidth-sweep size, and a 2^30 + 5 sort
that takes the 64-bit look-back status words) through the C ABI.

At these sizes the tests use properties that do not depend on N: sortedness,
a permutation check by scatter-count, exact key/value pairing by gather,
stability, wrap-around sums, scan differences. Where the oracle finishes in
seconds on a host copy (sums, Min/MaxLoc, histograms), results are compared
with it directly."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 1 << 28


def _u32_as_i64(t):
    import torch
    return t.view(torch.int32).to(torch.int64) & 0xFFFFFFFF


def _top16_counts(t64):
    import torch
    return torch.bincount(t64 >> 16, minlength=1 << 16)


@pytest.fixture(scope="module")
def gen():
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(2028)
    return g


def test_sort_u32_full_size(prims, gen):
    import torch
    x = torch.randint(-2 ** 31, 2 ** 31, (N,), generator=gen, device="cuda",
                      dtype=torch.int32).view(torch.uint32)
    xin = _u32_as_i64(x)
    out = torch.empty_like(x)
    prims.sort_copy(x, out)
    k = _u32_as_i64(out)
    assert bool((k[1:] >= k[:-1]).all())
    assert torch.equal(_top16_counts(k), _top16_counts(xin))
    assert int(k.sum()) == int(xin.sum())
    # descending, in place
    prims.sort(x, descending=True)
    kd = _u32_as_i64(x)
    assert bool((kd[1:] <= kd[:-1]).all())
    assert torch.equal(kd.flip(0), k)


def test_sort_u64_full_size(prims, gen):
    import torch
    x = torch.randint(-2 ** 63, 2 ** 63 - 1, (N,), generator=gen, device="cuda", dtype=torch.int64)
    flip = torch.tensor(-2 ** 63, dtype=torch.int64, device="cuda")
    xin = x.clone()
    prims.sort(x.view(torch.uint64))
    k = x ^ flip                          # unsigned order as signed order
    assert bool((k[1:] >= k[:-1]).all())
    top = lambda t: torch.bincount(((t ^ flip) >> 48) + 32768, minlength=1 << 16)  # noqa: E731
    assert torch.equal(top(x), top(xin))
    assert int(x.sum()) == int(xin.sum())   # wrap-around sums agree for a permutation


def test_sort_pairs_f32_i32_full_size_stable(prims, gen):
    import torch
    keys = torch.randn(N, generator=gen, device="cuda", dtype=torch.float32)
    keys[: N // 8] = torch.round(keys[: N // 8] * 4) / 4      # many equal keys
    vals = torch.arange(N, device="cuda", dtype=torch.int32)
    ko, vo = torch.empty_like(keys), torch.empty_like(vals)
    prims.sort_pairs_copy(keys, vals, ko, vo)
    assert bool((ko[1:] >= ko[:-1]).all())
    mark = torch.zeros(N, dtype=torch.int32, device="cuda")
    mark.index_add_(0, vo.long(), torch.ones_like(vo))
    assert bool((mark == 1).all())                              # values are a permutation
    assert torch.equal(keys[vo.long()].view(torch.int32), ko.view(torch.int32))  # exact pairing
    same = ko[1:].view(torch.int32) == ko[:-1].view(torch.int32)
    assert bool((vo[1:][same] > vo[:-1][same]).all())           # stable


def test_sort_wide_status_words(prims, gen):
    """n >= 2^30 switches the per-digit look-back to 64-bit status words."""
    import torch
    n = (1 << 30) + 5
    x = torch.randint(-2 ** 31, 2 ** 31, (n,), generator=gen, device="cuda",
                      dtype=torch.int32).view(torch.uint32)
    xin = _u32_as_i64(x)
    counts, total = _top16_counts(xin), int(xin.sum())
    del xin
    prims.sort(x)
    k = _u32_as_i64(x)
    assert bool((k[1:] >= k[:-1]).all())
    assert torch.equal(_top16_counts(k), counts)
    assert int(k.sum()) == total


def test_scans_full_size(prims, gen):
    import torch
    x = torch.randint(0, 1024, (N,), generator=gen, device="cuda", dtype=torch.int64)
    out = prims.exclusive_scan(x)
    assert int(out[0]) == 0
    assert torch.equal(out[1:] - out[:-1], x[:-1])
    assert int(out[-1] + x[-1]) == int(x.sum())
    # int32 inclusive with wrap-around (sums exceed 2^31)
    y = torch.randint(-2 ** 31, 2 ** 31, (N,), generator=gen, device="cuda", dtype=torch.int32)
    inc = prims.inclusive_scan(y)
    assert int(inc[0]) == int(y[0])
    assert torch.equal(inc[1:] - inc[:-1], y[1:])              # int32 arithmetic wraps
    # min / max scans are monotone and hit the running extreme
    mx = prims.inclusive_scan(y, op="maximum")
    assert bool((mx[1:] >= mx[:-1]).all()) and int(mx[-1]) == int(y.max())


def test_reductions_full_size(prims, orc, gen):
    import torch
    x = torch.rand(N, generator=gen, device="cuda", dtype=torch.float32) * 2 - 1
    xh = x.cpu().numpy()
    hi, _ = orc.exact_sum(xh)
    a = float(np.abs(xh.astype(np.float64)).sum())
    u32 = 2.0 ** -24
    assert abs(prims.reduce_sum(x) - hi) <= 64 * np.log2(N) * u32 * a
    assert abs(prims.reduce_sum(x, mode=1) - hi) <= 2.0 ** -50 * a
    assert prims.reduce_minloc(x) == orc.reduce_minloc(xh)
    assert prims.reduce_maxloc(x) == orc.reduce_maxloc(xh)
    d = torch.rand(N, generator=gen, device="cuda", dtype=torch.float64) * 2 - 1
    dh = d.cpu().numpy()
    assert prims.reduce_minloc(d) == orc.reduce_minloc(dh)
    assert prims.reduce_maxloc(d) == orc.reduce_maxloc(dh)
    dhi, _ = orc.exact_sum(dh)
    assert abs(prims.reduce_sum(d) - dhi) <= 64 * np.log2(N) * 2.0 ** -53 * float(np.abs(dh).sum())


def test_histogram_full_size(prims, orc, gen):
    import torch
    w = 1.0 / np.arange(1, 65537, dtype=np.float64) ** 1.1
    cdf = torch.from_numpy(np.cumsum(w) / w.sum()).cuda()
    u = torch.rand(N, generator=gen, device="cuda", dtype=torch.float64)
    z = torch.searchsorted(cdf, u, right=True).clamp_(0, 65535).to(torch.int32)
    del u
    zh = z.cpu().numpy()
    for nb in (256, 65536):
        zz = z if nb == 65536 else (z & 255)
        got = prims.histogram(zz, nb).cpu().numpy().astype(np.uint64)
        ref = orc.histogram(zh if nb == 65536 else (zh & 255), nb)
        np.testing.assert_array_equal(got, ref)
