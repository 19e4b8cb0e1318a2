"""Builds libpvdb.so (the sm_103a CUDA library behind include/pvdb.h) in-tree.

Every translation unit under csrc/ is compiled by nvcc in parallel with one
-gencode (compute_103a -> sm_103a) and linked into plenvdb_gb300/libpvdb.so
against the shared CUDA runtime. Objects go to plenvdb_gb300/_build/.
Rebuilds only what changed (source or shared header newer than the object).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpvdb.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "--expt-relaxed-constexpr", "-I", INCLUDE]


def nvcc() -> str:
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpvdb")


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers_mtime() -> float:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(INCLUDE, "pvdb.h"))
    return max(os.path.getmtime(h) for h in hs)


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(BUILD, src[:-3] + ".o")
    cmd = [nvcc(), *ARCH, *FLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> str:
    """Compile csrc/*.cu and link libpvdb.so; returns the library path."""
    extra = list(extra or [])
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    hdr = _headers_mtime()
    todo = []
    for s in srcs:
        obj = os.path.join(BUILD, s[:-3] + ".o")
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < max(
                hdr, os.path.getmtime(os.path.join(CSRC, s))):
            todo.append(s)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(todo), os.cpu_count() or 4))) as ex:
        for obj in ex.map(lambda s: _compile(s, extra), todo):
            if verbose:
                print("compiled", obj)
    objs = [os.path.join(BUILD, s[:-3] + ".o") for s in srcs]
    if todo or force or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        cmd = [nvcc(), *ARCH, "-shared", "-cudart", "shared", "-o", tmp, *objs]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
