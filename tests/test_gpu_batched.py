"""Batched WorkGroup loops, segmented scan / sort, CUDA graphs and batched
Jacobi sweeps through the C ABI, against the oracle applied loop by loop
(the reference composition: one forall / scan / sort per loop)."""
import numpy as np
import pytest

from conftest import to_dev, to_host

pytestmark = pytest.mark.gpu

U32 = 2.0 ** -24


def lognormal_lengths(rng, nloops, median, sigma, lo, hi):
    return np.clip(np.round(np.exp(rng.normal(np.log(median), sigma, nloops))), lo, hi).astype(np.int64)


def _loops(rng, lens):
    import torch
    xs = [torch.from_numpy(rng.uniform(-1, 1, int(n)).astype(np.float32)).cuda() for n in lens]
    ys = [torch.from_numpy(rng.uniform(-1, 1, int(n)).astype(np.float32)).cuda() for n in lens]
    px = torch.tensor([t.data_ptr() for t in xs], dtype=torch.int64, device="cuda")
    py = torch.tensor([t.data_ptr() for t in ys], dtype=torch.int64, device="cuda")
    return xs, ys, px, py


@pytest.mark.parametrize("autotune", [False, True])
def test_batched_axpy_sum_matches_per_loop_oracle(prims, orc, autotune):
    import torch
    rng = np.random.default_rng(11)
    lens = lognormal_lengths(rng, 300, 2000, 1.5, 32, 1 << 16)
    lens[5] = 0                     # an empty loop
    lens[7] = 1
    xs, ys, px, py = _loops(rng, lens)
    y0 = [t.cpu().numpy().copy() for t in ys]
    plan = prims.BatchPlan(lens)
    sums = torch.full((len(lens),), np.nan, dtype=torch.float64, device="cuda")
    reps = 1
    if autotune:
        # autotuning runs the loops several times (5 variants x 4 runs each)
        prims.batched_axpy_sum(plan, 0.5, px, py, sums, autotune=True)
        reps += 20
    prims.batched_axpy_sum(plan, 0.5, px, py, sums)
    got_sums = to_host(sums)
    for i, n in enumerate(lens):
        y = y0[i].copy()
        for _ in range(reps):
            orc.axpy(np.float32(0.5), xs[i].cpu().numpy(), y)
        gy = to_host(ys[i])
        np.testing.assert_allclose(gy, y, rtol=4 * reps * U32, atol=4 * reps * U32)
        exact, _ = orc.exact_sum(gy.astype(np.float32))
        bound = 1e-6 * float(np.abs(gy).sum()) + 1e-300
        assert abs(got_sums[i] - exact) <= bound, (i, n)
    info = plan.info()
    assert info["total"] == int(lens.sum()) and info["tiles"] > 0


@pytest.mark.parametrize("shape", [(256, 8), (256, 16), (512, 8), (128, 16), (256, 4)])
def test_batched_every_launch_shape_loop_by_loop(prims, orc, shape):
    """Each launch shape the autotuner picks from, pinned: loops carved from
    one flat array at odd offsets, an empty loop between long ones (its sum
    is 0), loops much longer than a block's run of tiles (their partials
    come from several blocks), and a run of one-element loops."""
    import torch
    rng = np.random.default_rng(23)
    lens = np.concatenate([lognormal_lengths(rng, 200, 3000, 1.2, 1, 1 << 17),
                           [0, 1 << 19, 0, 1, 1, 1, 3 * (1 << 18) + 5, 0]]).astype(np.int64)
    offs = np.concatenate([[0], np.cumsum(lens)]) + 3   # every loop starts off a 16-byte boundary
    total = int(offs[-1]) + 3
    x = rng.uniform(-1, 1, total).astype(np.float32)
    y = rng.uniform(-1, 1, total).astype(np.float32)
    dx, dy = to_dev(x), to_dev(y)
    px = torch.tensor([dx.data_ptr() + 4 * int(o) for o in offs[:-1]], dtype=torch.int64, device="cuda")
    py = torch.tensor([dy.data_ptr() + 4 * int(o) for o in offs[:-1]], dtype=torch.int64, device="cuda")
    plan = prims.BatchPlan(lens)
    plan.set_shape(*shape)
    info = plan.info()
    assert (info["block"], info["tile"]) == (shape[0], shape[0] * shape[1])
    sums = torch.full((len(lens),), np.nan, dtype=torch.float64, device="cuda")
    prims.batched_axpy_sum(plan, 0.25, px, py, sums)
    got_sums, gy = to_host(sums), to_host(dy)
    ref = y.copy()
    orc.axpy(np.float32(0.25), x[3:-3], ref[3:-3])
    np.testing.assert_allclose(gy, ref, rtol=4 * U32, atol=4 * U32)
    assert np.array_equal(gy[:3], y[:3]) and np.array_equal(gy[-3:], y[-3:])  # nothing outside the loops
    for i, n in enumerate(lens):
        seg = gy[offs[i]:offs[i + 1]]
        exact, lo = orc.exact_sum(seg)
        bound = 1e-6 * float(np.abs(seg).sum())
        assert abs((got_sums[i] - exact) - lo) <= bound, (shape, i, int(n), got_sums[i], exact)
        if n == 0:
            assert got_sums[i] == 0.0
    with pytest.raises(Exception):
        plan.set_shape(256, 3)
    plan.close()


def test_batched_full_workgroup_shape_loop_by_loop(prims, orc):
    """The batched-loops configuration at full size: 4096 loops with
    lognormal(median 2000, sigma 1.5) lengths clipped to [32, 2^20], carved
    from one flat array (so most loops start off a 16-byte boundary), fp32
    axpy plus a compensated per-loop sum.  Every loop is checked against the
    oracle, and the one-launch-per-loop schedule (the ordered WorkGroup
    runner's) gives the same results within the same bounds."""
    import ctypes as C

    import torch
    from raja_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(4)
    lens = lognormal_lengths(rng, 4096, 2000, 1.5, 32, 1 << 20)
    offs = np.concatenate([[0], np.cumsum(lens)])
    total = int(offs[-1])
    x = rng.uniform(-1, 1, total).astype(np.float32)
    y = rng.uniform(-1, 1, total).astype(np.float32)
    dx, dy, dy2 = to_dev(x), to_dev(y), to_dev(y)
    px = torch.tensor([dx.data_ptr() + 4 * int(o) for o in offs[:-1]], dtype=torch.int64, device="cuda")
    py = torch.tensor([dy.data_ptr() + 4 * int(o) for o in offs[:-1]], dtype=torch.int64, device="cuda")
    plan = prims.BatchPlan(lens)
    sums = torch.full((len(lens),), np.nan, dtype=torch.float64, device="cuda")
    prims.batched_axpy_sum(plan, 0.75, px, py, sums)
    # the same work as one launch per loop, issued from C++
    sums2 = torch.full((len(lens),), np.nan, dtype=torch.float64, device="cuda")
    hx = (C.c_void_p * len(lens))(*[dx.data_ptr() + 4 * int(o) for o in offs[:-1]])
    hy = (C.c_void_p * len(lens))(*[dy2.data_ptr() + 4 * int(o) for o in offs[:-1]])
    hl = (C.c_int64 * len(lens))(*[int(n) for n in lens])
    rc = lib.b200_loops_axpy_sum_f32(len(lens), hl, C.c_float(0.75), hx, hy, sums2.data_ptr(), 1,
                                     torch.cuda.current_stream().cuda_stream)
    assert rc == 0, lib.b200_last_error_string()
    prims.synchronize()
    yr = orc.axpy(np.float32(0.75), x, y.copy())
    gy, gy2 = to_host(dy), to_host(dy2)
    np.testing.assert_allclose(gy, yr, rtol=4 * U32, atol=4 * U32)
    assert np.array_equal(gy, gy2)                 # the same per-element arithmetic
    s1, s2 = to_host(sums), to_host(sums2)
    for i in range(len(lens)):
        seg = gy[offs[i]:offs[i + 1]]
        exact, lo = orc.exact_sum(seg)
        bound = 1e-6 * float(np.abs(seg).sum()) + 1e-300
        assert abs((s1[i] - exact) - lo) <= bound, (i, int(lens[i]))
        assert abs((s2[i] - exact) - lo) <= bound, (i, int(lens[i]))
    plan.close()


def test_loop_axpy_sum_single(prims, orc):
    import torch
    rng = np.random.default_rng(2)
    for n in (0, 1, 1000, 1 << 20):
        x = rng.uniform(-1, 1, n).astype(np.float32)
        y = rng.uniform(-1, 1, n).astype(np.float32)
        dx, dy = to_dev(x), to_dev(y)
        out = torch.zeros(1, dtype=torch.float64, device="cuda")
        prims.loop_axpy_sum(0.5, dx, dy, out)
        prims.synchronize()
        yr = orc.axpy(np.float32(0.5), x, y.copy())
        np.testing.assert_allclose(to_host(dy), yr, rtol=4 * U32, atol=4 * U32)
        exact, _ = orc.exact_sum(to_host(dy))
        assert abs(out.item() - exact) <= 1e-6 * float(np.abs(yr).sum()) + 1e-300


def pareto_lengths(rng, nseg, alpha=1.5, xmin=32, cap=1 << 20):
    return np.minimum(np.floor(xmin * (1 - rng.random(nseg)) ** (-1 / alpha)), cap).astype(np.int64)


def test_segmented_scans_bit_exact(prims, orc):
    rng = np.random.default_rng(3)
    lens = pareto_lengths(rng, 2000)
    lens[:3] = [0, 1, 0]            # empty and single-element segments
    plan = prims.BatchPlan(lens)
    x = rng.integers(-(1 << 20), 1 << 20, plan.total).astype(np.int32)
    d = to_dev(x)
    inc = to_host(prims.segmented_inclusive_scan(plan, d))
    exc = to_host(prims.segmented_exclusive_scan(plan, d))
    for i in range(len(lens)):
        a, b = plan.offsets[i], plan.offsets[i + 1]
        seg = x[a:b]
        np.testing.assert_array_equal(inc[a:b], orc.scan(seg, "plus"), err_msg=f"seg {i}")
        np.testing.assert_array_equal(exc[a:b], orc.scan(seg, "plus", exclusive=True, init=0),
                                      err_msg=f"seg {i}")


def test_segmented_sort_bit_exact(prims, orc):
    rng = np.random.default_rng(4)
    lens = pareto_lengths(rng, 3000)
    lens[10] = 9000                 # longer than the per-block sort: radix path
    lens[11] = 4096
    lens[12] = 4097
    plan = prims.BatchPlan(lens)
    k = rng.integers(0, 2 ** 32, plan.total, dtype=np.uint64).astype(np.uint32)
    for desc in (False, True):
        d = to_dev(k)
        prims.segmented_sort(plan, d, descending=desc)
        got = to_host(d)
        for i in range(len(lens)):
            a, b = plan.offsets[i], plan.offsets[i + 1]
            np.testing.assert_array_equal(got[a:b], orc.sort(k[a:b], descending=desc),
                                          err_msg=f"seg {i} desc={desc}")


@pytest.mark.parametrize("case", ["over_256_long_segments", "long_segments_sorted_one_by_one"])
def test_segmented_sort_long_segment_paths(prims, orc, case):
    """Long segments (more than 4096 keys) are sorted together as
    (segment << 32 | key) in one 64-bit sort when there are several of
    moderate length -- here more than 256 of them, so the segment bits reach
    past the low byte of the high word -- and one sort call per segment when
    they are long; keys with many duplicates, both directions, against the
    oracle segment by segment."""
    rng = np.random.default_rng(9)
    if case == "over_256_long_segments":
        lens = np.empty(600, dtype=np.int64)
        lens[0::2] = 4097 + rng.integers(0, 700, 300)
        lens[1::2] = rng.integers(0, 50, 300)
    else:
        lens = np.array([5, 600000, 3, 700000, 10, 0], dtype=np.int64)
    plan = prims.BatchPlan(lens)
    k = rng.integers(0, 1000, plan.total, dtype=np.uint64).astype(np.uint32)
    k[::7] = rng.integers(0, 2 ** 32, k[::7].size, dtype=np.uint64).astype(np.uint32)
    for desc in (False, True):
        d = to_dev(k)
        prims.segmented_sort(plan, d, descending=desc)
        got = to_host(d)
        for i in range(len(lens)):
            a, b = plan.offsets[i], plan.offsets[i + 1]
            np.testing.assert_array_equal(got[a:b], orc.sort(k[a:b], descending=desc),
                                          err_msg=f"{case} seg {i} desc={desc}")
    plan.close()


def test_graph_capture_replays_batched_sweeps(prims):
    import torch
    rng = np.random.default_rng(5)
    lens = lognormal_lengths(rng, 64, 2000, 1.0, 32, 1 << 14)
    xs, ys, px, py = _loops(rng, lens)
    plan = prims.BatchPlan(lens)
    sums = torch.zeros(len(lens), dtype=torch.float64, device="cuda")
    ref = [t.clone() for t in ys]
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        prims.batched_axpy_sum(plan, 0.25, px, py, sums, stream=stream)   # warm-up (no capture)
        stream.synchronize()
        g = prims.Graph(stream)
        with g:
            for _ in range(3):
                prims.batched_axpy_sum(plan, 0.25, px, py, sums, sync=False, stream=stream)
        for _ in range(2):
            g.launch()
        prims.synchronize(stream)
    for i in range(len(lens)):
        expect = ref[i] + 0.25 * xs[i] * 7            # 1 warm-up + 2 x 3 captured
        assert torch.allclose(ys[i], expect, rtol=1e-5, atol=1e-5)
    g.close()


def _meshes(rng, shapes):
    total = sum(a * b * c for a, b, c in shapes)
    u = rng.uniform(0, 1, total)
    return u


def test_jacobi_batched_bit_exact_vs_oracle(prims, orc):
    import torch
    rng = np.random.default_rng(6)
    shapes = [(int(a), int(b), int(c)) for a, b, c in rng.integers(3, 40, (40, 3))]
    shapes += [(3, 3, 3), (64, 5, 7)]
    plan = prims.JacobiPlan(shapes)
    u = _meshes(rng, shapes)
    f = rng.uniform(-1e-3, 1e-3, u.size)
    for use_f in (False, True):
        du, dn = to_dev(u), to_dev(u.copy())
        df = to_dev(f) if use_f else None
        resid = torch.zeros(len(shapes), dtype=torch.float64, device="cuda")
        prims.jacobi_sweep(plan, du, dn, resid, f=df)
        got, gres = to_host(dn), to_host(resid)
        for m, sh in enumerate(shapes):
            a, b = plan.offsets[m], plan.offsets[m + 1]
            ref = u[a:b].copy()
            r = orc.jacobi_sweep(u[a:b].copy(), ref, f[a:b].copy() if use_f else None, sh)
            np.testing.assert_array_equal(got[a:b], ref, err_msg=f"mesh {m} {sh}")
            assert gres[m] == r, (m, sh)


def test_jacobi_single_mesh_and_graph(prims, orc):
    import torch
    rng = np.random.default_rng(7)
    sh = (33, 17, 9)
    u = rng.uniform(0, 1, sh[0] * sh[1] * sh[2])
    du, dn = to_dev(u), to_dev(u.copy())
    resid = torch.zeros(1, dtype=torch.float64, device="cuda")
    prims.jacobi_mesh_sweep(sh, du, dn, resid)
    ref = u.copy()
    r = orc.jacobi_sweep(u.copy(), ref, None, sh)
    np.testing.assert_array_equal(to_host(dn), ref)
    assert resid.item() == r
    # 20 ping-pong sweeps captured in one graph match 20 oracle sweeps
    plan = prims.JacobiPlan([sh])
    stream = torch.cuda.Stream()
    a, b = to_dev(u), to_dev(u.copy())
    res = torch.zeros(20, dtype=torch.float64, device="cuda")
    with torch.cuda.stream(stream):
        prims.jacobi_sweep(plan, a, b, res[0:1], stream=stream)          # warm-up
        a.copy_(torch.from_numpy(u).cuda()); b.copy_(a)
        stream.synchronize()
        g = prims.Graph(stream)
        with g:
            for s in range(20):
                src, dst = (a, b) if s % 2 == 0 else (b, a)
                prims.jacobi_sweep(plan, src, dst, res[s:s + 1], sync=False, stream=stream)
        g.launch()
        prims.synchronize(stream)
    x, y = u.copy(), u.copy()
    rs = []
    for s in range(20):
        src, dst = (x, y) if s % 2 == 0 else (y, x)
        rs.append(orc.jacobi_sweep(src, dst, None, sh))
    np.testing.assert_array_equal(to_host(a), x)   # 20 sweeps: result back in a
    np.testing.assert_array_equal(to_host(res), np.array(rs))
    g.close()
