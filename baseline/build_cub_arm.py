"""Build recipe for the CUB comparison arm (benchmark only).

Compiles baseline/cub_arm.cu -- thin calls into the CUB that ships with the
CUDA toolkit, the library RAJA's CUDA scan and sort call -- into
baseline/libcubarm.so for sm_103a.  bench.py loads it to time CUB beside the
library's own scan and sort; nothing in the product links it.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cub_arm.cu")
OUT = os.path.join(HERE, "libcubarm.so")


def build(force: bool = False) -> str:
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= os.path.getmtime(SRC):
        return OUT
    nvcc = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cmd = [nvcc, "-O3", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
           "-Xcompiler", "-fPIC", "-shared", "-cudart", "shared", "-o", OUT + ".tmp", SRC]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {SRC}:\n{r.stdout}\n{r.stderr}")
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
