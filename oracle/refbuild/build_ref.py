"""Build recipe for oracle/_ref/ref_driver -- RAJA's own host policies.

Compiles oracle/refbuild/ref_driver.cpp and the reference's
src/PluginStrategy.cpp with g++ straight from the RAJA source tree (read in
place, never copied), with the hand-written RAJA/config.hpp and the
clean-room camp subset under oracle/refbuild/ first on the include path.
No CMake and no RAJA build system is involved.  The binary goes to
oracle/_ref/ (git-ignored).  Test infrastructure only: it produces the
reference fixtures under tests/golden/ and is never part of the product.

    python oracle/refbuild/build_ref.py [--ref /path/to/RAJA] [--force]

The compat front-end build (--compat) compiles the same driver source
against include/raja_compat instead, to check the front-end's seq/omp
semantics against those fixtures; it needs no reference tree.
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
ROOT = os.path.dirname(ORACLE)
OUT_DIR = os.path.join(ORACLE, "_ref")
REF_BIN = os.path.join(OUT_DIR, "ref_driver")
COMPAT_BIN = os.path.join(OUT_DIR, "compat_driver")
DRIVER = os.path.join(HERE, "ref_driver.cpp")
DEFAULT_REF = "/root/reference"

FLAGS = ["-std=c++17", "-O2", "-fopenmp", "-ffp-contract=off"]


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build_ref(ref: str = DEFAULT_REF, force: bool = False) -> str:
    inc = os.path.join(ref, "include")
    plugin = os.path.join(ref, "src", "PluginStrategy.cpp")
    if not os.path.isdir(inc):
        raise FileNotFoundError(f"RAJA source tree not found at {ref}")
    deps = [DRIVER] + [os.path.join(HERE, d, f) for d in ("camp", "camp/list", "RAJA")
                       for f in os.listdir(os.path.join(HERE, d))
                       if f.endswith(".hpp")]
    if not force and not _stale(REF_BIN, deps):
        return REF_BIN
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = ["g++"] + FLAGS + ["-I", HERE, "-I", inc, DRIVER, plugin, "-o", REF_BIN + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(REF_BIN + ".tmp", REF_BIN)
    return REF_BIN


def build_compat(force: bool = False) -> str:
    inc = os.path.join(ROOT, "include", "raja_compat")
    hdr = os.path.join(inc, "RAJA", "RAJA.hpp")
    if not force and not _stale(COMPAT_BIN, [DRIVER, hdr]):
        return COMPAT_BIN
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = ["g++"] + FLAGS + ["-I", inc, DRIVER, "-o", COMPAT_BIN + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(COMPAT_BIN + ".tmp", COMPAT_BIN)
    return COMPAT_BIN


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=DEFAULT_REF)
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--compat", action="store_true")
    a = ap.parse_args()
    print(build_compat(a.force) if a.compat else build_ref(a.ref, a.force))
    sys.exit(0)
