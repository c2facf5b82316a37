"""The C++ layer: the raja_compat front-end on the host (CPU), and RAJA-API
programs on the b200 policies against seq_exec (GPU)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = [f"-I{ROOT}/include/raja_compat", f"-I{ROOT}/include"]


def _run(cmd, **kw):
    r = subprocess.run(cmd, capture_output=True, text=True, **kw)
    return r


def test_compat_front_end_host(tmp_path):
    exe = str(tmp_path / "test_raja_compat")
    r = _run(["g++", "-std=c++17", "-O1", "-fopenmp", *INC, f"{ROOT}/tests/cpp/test_raja_compat.cpp", "-o", exe])
    assert r.returncode == 0, r.stderr[-3000:]
    r = _run([exe])
    assert r.returncode == 0, r.stdout[-3000:]
    assert "FAIL" not in r.stdout


@pytest.mark.gpu
def test_b200_policies_against_seq(tmp_path):
    import raja_gb300.build as b
    lib = b.build()
    nvcc = b.nvcc()
    exe = str(tmp_path / "test_raja_b200")
    r = _run([nvcc, "-std=c++17", "--extended-lambda", "--expt-relaxed-constexpr", "-O2", "-DRAJA_ENABLE_NVTX",
              *b.ARCH, *INC,
              f"{ROOT}/tests/cpp/test_raja_b200.cu", "-o", exe, f"-L{os.path.dirname(lib)}", "-lb200prims",
              f"-Xlinker", f"-rpath={os.path.dirname(lib)}"])
    assert r.returncode == 0, r.stderr[-4000:]
    r = _run([exe], timeout=600)
    print(r.stdout)
    assert "FAIL" not in r.stdout, r.stdout[-6000:]
    assert r.returncode == 0
