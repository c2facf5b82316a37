"""The b200 policies bind to RAJA's own extension points.

tests/cpp/reference_binding.cu is a RAJA application whose policy alias
switches from seq_exec to b200_exec.  It is compiled here with nvcc against
an installed RAJA -- the reference's unmodified headers, with the
hand-written config and the clean-room camp subset of oracle/refbuild/ --
plus include/raja_b200/RAJA_b200.hpp, and linked with libb200prims and the
reference's src/PluginStrategy.cpp.  RAJA's forall (ranges and IndexSets),
ReduceSum / ReduceMinLoc on b200_reduce, expt::Reduce params, scans, sorts
and WorkPool / WorkGroup (b200_work, through detail::WorkRunner) must all
resolve to b200 overloads for it to build.  The program then
runs: its seq_exec half always, and its b200 half, checked against seq_exec,
where a CUDA device is present.  The test needs the reference tree (not
present on the GPU host) and skips without it.
"""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_b200_binds_to_raja_extension_points(tmp_path):
    from oracle.refbuild import build_ref
    ref = build_ref.DEFAULT_REF
    if not os.path.isdir(os.path.join(ref, "include", "RAJA")):
        pytest.skip("the RAJA source tree is not available here")
    import raja_gb300.build as b
    lib = b.build()
    exe = str(tmp_path / "reference_binding")
    cmd = [b.nvcc(), "-std=c++17", "--extended-lambda", "--expt-relaxed-constexpr", "-O2", *b.ARCH,
           "-I", os.path.join(ROOT, "oracle", "refbuild"), "-I", os.path.join(ref, "include"),
           "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "reference_binding.cu"),
           os.path.join(ref, "src", "PluginStrategy.cpp"), "-o", exe,
           f"-L{os.path.dirname(lib)}", "-lb200prims", "-Xlinker", f"-rpath={os.path.dirname(lib)}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
    assert "FAIL" not in r.stdout
