"""Small case for profiling one onesweep pass: two 64-bit key sorts of
2^25 uniform keys (256 MB each way, above the 129 MB L2) through the C ABI.
Used by the ncu commands quoted in this folder; prints nothing but 'ok'."""
import os
import sys

import torch

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import raja_gb300 as rg  # noqa: E402

n = 1 << 25
g = torch.Generator(device="cuda")
g.manual_seed(0)
x = torch.randint(-2 ** 63, 2 ** 63 - 1, (n,), device="cuda", dtype=torch.int64,
                  generator=g).view(torch.uint64)
y = torch.empty_like(x)
for _ in range(2):
    rg.sort_copy(x, y)
torch.cuda.synchronize()
print("ok")
