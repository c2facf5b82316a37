"""Small, self-contained workloads for ncu captures of single kernels.

Run from the repository root:

    python tests/profile_cases.py sort_pass
        two 64-bit key sorts of 2^25 uniform keys (256 MB each way, above the
        129 MB L2) through the C ABI: 18 launches (histogram plus 8 onesweep
        passes per sort).
    python tests/profile_cases.py sort_k32_n2p27 | sort_k64_n2p27 | sort_pairs_n2p27
        one sort of 2^27 uniform 32-bit keys, 64-bit keys, or normal f32 keys
        with int32 index values (0.5-1 GB per array, several times the L2).
    python tests/profile_cases.py scan_i64_n2p27
        two int64 exclusive scans of 2^27 elements uniform in {0..1023}
        (1 GB in, 1 GB out).
    python tests/profile_cases.py jacobi_mesh512
        three fused Jacobi sweeps of one 512^3 fp64 mesh (two 1.07 GB
        buffers).
    python tests/profile_cases.py batched_4096_loops
        the 4096-loop WorkGroup shape (lognormal lengths, median 2000,
        sigma 1.5, 2.4e7 elements): one autotuned persistent fp32 axpy +
        per-loop compensated sum, then two more launches of it.

Each prints "ok" and nothing else.  The summaries under profiles/ quote the
ncu commands that use them.
"""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import torch  # noqa: E402

import raja_gb300 as rg  # noqa: E402


def _gen(seed):
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    return g


def sort_pass():
    n = 1 << 25
    x = torch.randint(-2 ** 63, 2 ** 63 - 1, (n,), device="cuda", dtype=torch.int64,
                      generator=_gen(0)).view(torch.uint64)
    y = torch.empty_like(x)
    for _ in range(2):
        rg.sort_copy(x, y)


def sort_k32_n2p27():
    n = 1 << 27
    x = torch.randint(-2 ** 31, 2 ** 31, (n,), device="cuda", dtype=torch.int32,
                      generator=_gen(0)).view(torch.uint32)
    rg.sort_copy(x, torch.empty_like(x))


def sort_k64_n2p27():
    n = 1 << 27
    x = torch.randint(-2 ** 63, 2 ** 63 - 1, (n,), device="cuda", dtype=torch.int64,
                      generator=_gen(0)).view(torch.uint64)
    rg.sort_copy(x, torch.empty_like(x))


def sort_pairs_n2p27():
    n = 1 << 27
    k = torch.randn(n, device="cuda", dtype=torch.float32, generator=_gen(0))
    v = torch.arange(n, device="cuda", dtype=torch.int32)
    rg.sort_pairs(k, v)


def scan_i64_n2p27():
    n = 1 << 27
    x = torch.randint(0, 1024, (n,), device="cuda", dtype=torch.int64, generator=_gen(0))
    out = torch.empty_like(x)
    for _ in range(2):
        rg.exclusive_scan(x, out=out)


def jacobi_mesh512():
    plan = rg.JacobiPlan([(512, 512, 512)])
    u = torch.rand(plan.total, dtype=torch.float64, device="cuda", generator=_gen(1))
    un = u.clone()
    r = torch.zeros(1, dtype=torch.float64, device="cuda")
    for sw in range(3):
        a, b = (u, un) if sw % 2 == 0 else (un, u)
        rg.jacobi_sweep(plan, a, b, r)
    plan.close()


def batched_4096_loops():
    import numpy as np
    rng = np.random.default_rng(4)
    lens = np.clip(np.round(np.exp(rng.normal(np.log(2000), 1.5, 4096))), 32, 1 << 20).astype(np.int64)
    offs = np.concatenate([[0], np.cumsum(lens)])
    x = torch.rand(int(offs[-1]), device="cuda", generator=_gen(2)) * 2 - 1
    y = torch.rand(int(offs[-1]), device="cuda", generator=_gen(3)) * 2 - 1
    px = torch.tensor([x.data_ptr() + 4 * int(o) for o in offs[:-1]], dtype=torch.int64, device="cuda")
    py = torch.tensor([y.data_ptr() + 4 * int(o) for o in offs[:-1]], dtype=torch.int64, device="cuda")
    sums = torch.zeros(len(lens), dtype=torch.float64, device="cuda")
    plan = rg.BatchPlan(lens)
    rg.batched_axpy_sum(plan, 1e-3, px, py, sums, autotune=True)
    for _ in range(2):
        rg.batched_axpy_sum(plan, 1e-3, px, py, sums)
    plan.close()


CASES = {f.__name__: f for f in (sort_pass, sort_k32_n2p27, sort_k64_n2p27, sort_pairs_n2p27,
                                 scan_i64_n2p27, jacobi_mesh512, batched_4096_loops)}

if __name__ == "__main__":
    if len(sys.argv) != 2 or sys.argv[1] not in CASES:
        sys.exit("usage: python tests/profile_cases.py {" + ",".join(CASES) + "}")
    CASES[sys.argv[1]]()
    torch.cuda.synchronize()
    print("ok")
