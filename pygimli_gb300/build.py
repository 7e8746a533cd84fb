"""Build libertgb.so in-tree (pygimli_gb300/_lib/) with nvcc for sm_103a.

Each translation unit of pygimli_gb300/csrc is compiled in parallel, then
linked with the static CUDA runtime.  ``python -m pygimli_gb300.build``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libertgb.so")
SOURCES = ["setup.cpp", "assemble.cu", "pcg.cu", "pcg_mixed.cu", "fsai.cu", "jacobian.cu", "capi.cu", "noalloc.cu", "learned.cu", "batch.cu", "cgls.cu", "refine.cu", "complex.cu", "ic0.cu", "band.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fno-strict-aliasing"]


def nvcc():
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _compile(src, obj, extra):
    cmd = [nvcc(), *FLAGS, *ARCH, *extra, "-c", "-x", "cu", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose=False, extra=()):
    os.makedirs(OUT_DIR, exist_ok=True)
    objdir = os.path.join(OUT_DIR, "obj")
    os.makedirs(objdir, exist_ok=True)
    newest_src = max(os.path.getmtime(os.path.join(CSRC, f)) for f in os.listdir(CSRC))
    hdr = os.path.join(os.path.dirname(HERE), "include", "ertgb.h")
    newest_src = max(newest_src, os.path.getmtime(hdr))
    if os.path.exists(LIB) and os.path.getmtime(LIB) > newest_src and not extra:
        return LIB
    objs = [os.path.join(objdir, s + ".o") for s in SOURCES]
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        list(ex.map(lambda so: _compile(so[0], so[1], list(extra)), zip(SOURCES, objs)))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared", *ARCH, "-o", tmp, *objs, "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra=tuple(sys.argv[1:]))
