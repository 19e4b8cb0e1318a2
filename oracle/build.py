"""Build recipe of the CPU oracle (test infrastructure only).

* oracle/_build/liboracle.so — the C++ restatement (pvdb_oracle.cpp), built
  anywhere (here and on the GPU machine) with g++ -fopenmp -ffp-contract=off.
* oracle/_ref/libnanoref.so — the reference harness (ref_harness.cpp), which
  includes the reference's own header-only NanoVDB (NanoVDB.h + GridBuilder.h)
  from the mounted reference tree. Built only where that tree exists; its
  outputs stay in oracle/_ref/ (git-ignored).
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(BUILD, "liboracle.so")
REF_LIB = os.path.join(REF_OUT, "libnanoref.so")
REFERENCE_ROOT = "/root/reference"
NANOVDB_INC = os.path.join(REFERENCE_ROOT, "openvdb", "nanovdb")

CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math"]


def _newer(src: str, out: str) -> bool:
    return not os.path.exists(out) or os.path.getmtime(out) < os.path.getmtime(src)


def build_oracle(force: bool = False) -> str:
    src = os.path.join(HERE, "pvdb_oracle.cpp")
    os.makedirs(BUILD, exist_ok=True)
    if force or _newer(src, LIB):
        tmp = LIB + ".tmp"
        cmd = ["g++", *CXXFLAGS, "-fopenmp", src, "-o", tmp]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode:
            raise RuntimeError(f"oracle build failed:\n{res.stderr}")
        os.replace(tmp, LIB)
    return LIB


def build_ref(force: bool = False) -> str | None:
    """Compile the NanoVDB reference harness when the reference tree is mounted."""
    if not os.path.exists(os.path.join(NANOVDB_INC, "nanovdb", "NanoVDB.h")):
        return None
    src = os.path.join(HERE, "ref_harness.cpp")
    os.makedirs(REF_OUT, exist_ok=True)
    if force or _newer(src, REF_LIB):
        tmp = REF_LIB + ".tmp"
        cmd = ["g++", *CXXFLAGS, "-I", NANOVDB_INC, src, "-o", tmp, "-lpthread"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode:
            raise RuntimeError(f"reference harness build failed:\n{res.stderr}")
        os.replace(tmp, REF_LIB)
    return REF_LIB


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
