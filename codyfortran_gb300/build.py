"""Builds the in-tree CUDA library libcodygpu.so for sm_103a.

Each translation unit is compiled by nvcc in parallel, then linked into
codyfortran_gb300/_build/libcodygpu.so.  Re-running is incremental (object
files newer than their sources and headers are reused).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(OUT_DIR, "libcodygpu.so")
SOURCES = ["ctx.cu", "k_onebody.cu", "k_ci.cu", "k_mf.cu", "k_lanczos.cu", "noalloc.cu", "k_tc.cu", "k_fx.cu", "k_mixed.cu", "k_adjoint.cu", "autotune.cu", "k_sys.cu", "k_adjoint_mc.cu"]
HEADERS = ["common.cuh", "tc.cuh", "dfloat.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libcodygpu.so")


def _newest_dep() -> float:
    deps = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "cody_gpu.h")]
    return max(os.path.getmtime(p) for p in deps)


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(path), _newest_dep()):
        return obj
    cmd = [_nvcc(), *ARCH, *FLAGS, *extra, "-I", os.path.join(ROOT, "include"), "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, extra: list[str] | None = None) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    extra = extra or []
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [_nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
