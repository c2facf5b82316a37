"""Small, self-contained workloads for ncu captures of single kernels.

    python -m raja_gb300.profile_cases sort_pass
        two 64-bit key sorts of 2^25 uniform keys (256 MB each way, above the
        129 MB L2) through the C ABI: 18 launches (histogram plus 8 onesweep
        passes per sort).
    python -m raja_gb300.profile_cases jacobi_mesh512
        three fused Jacobi sweeps of one 512^3 fp64 mesh (two 1.07 GB
        buffers).

Each prints "ok" and nothing else.  The summaries under profiles/ quote the
ncu commands that use them.
"""
import sys

import torch

import raja_gb300 as rg


def sort_pass():
    n = 1 << 25
    g = torch.Generator(device="cuda")
    g.manual_seed(0)
    x = torch.randint(-2 ** 63, 2 ** 63 - 1, (n,), device="cuda", dtype=torch.int64,
                      generator=g).view(torch.uint64)
    y = torch.empty_like(x)
    for _ in range(2):
        rg.sort_copy(x, y)


def jacobi_mesh512():
    plan = rg.JacobiPlan([(512, 512, 512)])
    g = torch.Generator(device="cuda")
    g.manual_seed(1)
    u = torch.rand(plan.total, dtype=torch.float64, device="cuda", generator=g)
    un = u.clone()
    r = torch.zeros(1, dtype=torch.float64, device="cuda")
    for sw in range(3):
        a, b = (u, un) if sw % 2 == 0 else (un, u)
        rg.jacobi_sweep(plan, a, b, r)
    plan.close()


CASES = {"sort_pass": sort_pass, "jacobi_mesh512": jacobi_mesh512}

if __name__ == "__main__":
    if len(sys.argv) != 2 or sys.argv[1] not in CASES:
        sys.exit("usage: python -m raja_gb300.profile_cases {" + ",".join(CASES) + "}")
    CASES[sys.argv[1]]()
    torch.cuda.synchronize()
    print("ok")
