"""Builds liblc2.so (CUDA, sm_103a) in-tree with nvcc.

The library is plain CUDA C++ behind a C ABI (include/lc2.h); it does not
link against PyTorch. Output: lc2registration_gb300/_build/liblc2.so.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(OUT_DIR, "liblc2.so")
SOURCES = ["lc2_capi.cu", "lc2_fused_f32.cu", "lc2_fused_f16.cu", "lc2_fused_bf16.cu",
           "lc2_list_f32.cu", "lc2_list_f16.cu", "lc2_list_bf16.cu", "lc2_fixed_f32.cu",
           "lc2_fixed_f16.cu", "lc2_fixed_bf16.cu", "lc2_ps_f32.cu", "lc2_ps_f16.cu",
           "lc2_ps_bf16.cu", "lc2_noalloc.cu",
           "lc2_export.cu", "lc2_optim.cpp", "lc2_serve.cpp", "lc2_stack_reg.cpp"]
DEPS = SOURCES + ["lc2_kernels.cuh", "lc2_fused.cuh", "lc2_fused_ws.cuh", "lc2_list.cuh",
                   "lc2_mi.cuh", "lc2_fused_fixed.cuh", "lc2_fused_ps.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the LC2 CUDA library cannot be built")


def needs_build() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    deps = [os.path.join(CSRC, d) for d in DEPS] + [os.path.join(ROOT, "include", "lc2.h")]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile each translation unit in parallel, then link liblc2.so."""
    if not force and not needs_build():
        return LIB_PATH
    os.makedirs(OUT_DIR, exist_ok=True)
    common = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "-I", os.path.join(ROOT, "include")]
    procs, objs = [], []
    for src in SOURCES:
        obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
        cmd = common + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((src, subprocess.Popen(cmd)))
        objs.append(obj)
    failed = [src for src, p in procs if p.wait() != 0]
    if failed:
        raise RuntimeError(f"nvcc failed on {failed}")
    tmp = LIB_PATH + ".tmp"
    subprocess.run([nvcc(), *ARCH, "-shared", "-o", tmp] + objs, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
