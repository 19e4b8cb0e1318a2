"""Build recipe of the CPU oracle (test infrastructure only).

* oracle/_build/liboracle.so — the C++ restatement (pvdb_oracle.cpp), built
  anywhere (here and on the GPU machine) with g++ -fopenmp -ffp-contract=off.
* oracle/_ref/libnanoref.so — the reference harness (ref_harness.cpp), which
  includes the reference's own header-only NanoVDB (NanoVDB.h + GridBuilder.h)
  from the mounted reference tree. Built only where that tree exists; its
  outputs stay in oracle/_ref/ (git-ignored).
* oracle/_ref/dvgo_ext/ — the reference's DirectVoxGO torch-extension sources
  (lib/cuda/render_utils*, total_variation*, adam_upd*), staged unmodified from
  the mounted reference tree so that they can be JIT-compiled on a machine with
  a GPU (load_dvgo_ext), where tests/golden/make_dvgo_ext_golden.py runs them to
  write golden vectors. Staged only where the tree exists; git-ignored.

The reference tree is found at $PVDB_REFERENCE_ROOT (default /root/reference).
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(BUILD, "liboracle.so")
REF_LIB = os.path.join(REF_OUT, "libnanoref.so")
REFERENCE_ROOT = os.environ.get("PVDB_REFERENCE_ROOT", "/root/reference")
NANOVDB_INC = os.path.join(REFERENCE_ROOT, "openvdb", "nanovdb")
DVGO_CUDA = os.path.join(REFERENCE_ROOT, "plenvdb", "lib", "cuda")
DVGO_STAGE = os.path.join(REF_OUT, "dvgo_ext")
# extension name -> its two source files (grid.py:17-29, masked_adam.py:11-15)
DVGO_EXTS = {
    "render_utils_cuda": ["render_utils.cpp", "render_utils_kernel.cu"],
    "total_variation_cuda": ["total_variation.cpp", "total_variation_kernel.cu"],
    "adam_upd_cuda": ["adam_upd.cpp", "adam_upd_kernel.cu"],
}

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
    """Compile the NanoVDB reference harness and stage the DirectVoxGO
    extension sources when the reference tree is mounted."""
    stage_dvgo_ext()
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


def stage_dvgo_ext() -> str | None:
    """Copy the reference's torch-extension sources, unmodified, into
    oracle/_ref/dvgo_ext/ (git-ignored). Returns the folder, or None when the
    reference tree is not mounted."""
    if not os.path.isdir(DVGO_CUDA):
        return DVGO_STAGE if os.path.isdir(DVGO_STAGE) else None
    os.makedirs(DVGO_STAGE, exist_ok=True)
    for files in DVGO_EXTS.values():
        for f in files:
            src, dst = os.path.join(DVGO_CUDA, f), os.path.join(DVGO_STAGE, f)
            if _newer(src, dst):
                shutil.copyfile(src, dst)
    return DVGO_STAGE


def _torch_lacks_deprecated_dispatch() -> bool:
    """True when this PyTorch's dispatch headers no longer take tensor.type()
    (the reference's AT_DISPATCH_FLOATING_TYPES(x.type(), ...) form)."""
    import torch
    inc = os.path.join(os.path.dirname(torch.__file__), "include")
    pat = re.compile(r"scalar_type\(\s*const\s+at::DeprecatedTypeProperties")
    for sub in ("ATen/Dispatch.h", "torch/headeronly/core/Dispatch.h", "ATen/Dispatch_v2.h"):
        p = os.path.join(inc, sub)
        if os.path.exists(p) and pat.search(open(p, errors="ignore").read()):
            return False
    return True


def load_dvgo_ext(name: str, build_root: str | None = None):
    """JIT-compile (torch.utils.cpp_extension) one staged reference extension
    for sm_103a and import it. Needs the CUDA toolkit; runs on the GPU machine."""
    from torch.utils.cpp_extension import load
    if not os.path.isdir(DVGO_STAGE):
        raise RuntimeError("reference extension sources are not staged (oracle/_ref/dvgo_ext)")
    os.environ.setdefault("TORCH_CUDA_ARCH_LIST", "10.0")
    build_dir = os.path.join(build_root or os.path.join(REF_OUT, "dvgo_build"), name)
    os.makedirs(build_dir, exist_ok=True)
    cuda_flags = ["-gencode", "arch=compute_103a,code=sm_103a"]
    if _torch_lacks_deprecated_dispatch():
        cuda_flags = ["-include", os.path.join(HERE, "dvgo_ext_compat.h"), *cuda_flags]
    srcs = [os.path.join(DVGO_STAGE, f) for f in DVGO_EXTS[name]]
    return load(name=name, sources=srcs, build_directory=build_dir,
                extra_cuda_cflags=cuda_flags, verbose=False)


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
