"""Builds libgbp.so (the CUDA library behind include/gbp.h) in-tree.

    python -m shiokaze_gb300.build [--force]

Every translation unit is compiled for sm_103a only
(-gencode arch=compute_103a,code=sm_103a), in parallel, then linked into
shiokaze_gb300/libgbp.so with the CUDA runtime linked statically. Sources
listed in FMAD_OFF are compiled with --fmad=false so their arithmetic rounds
like the reference's scalar C++.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgbp.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["setup_kernels.cu", "cg_kernels.cu", "mg_kernels.cu", "batch_kernels.cu", "gbp_batch.cpp",
           "gbp_solver.cpp", "gbp_api.cpp", "gbp_noalloc.cu", "csr_solver.cu",
           "advect_kernels.cu", "brick_kernels.cu"]
FMAD_OFF = {"setup_kernels.cu", "advect_kernels.cu"}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags(src: str) -> list[str]:
    f = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include"), "-I", CSRC,
         *ARCH]
    if src.endswith(".cu"):
        f += ["--extended-lambda", "-Xptxas", "-v"] if os.environ.get("GBP_PTXAS_VERBOSE") else ["--extended-lambda"]
        if src in FMAD_OFF:
            f.append("--fmad=false")
    return f


def _compile(src: str) -> str:
    obj = os.path.join(BUILD, src + ".o")
    path = os.path.join(CSRC, src)
    deps = [path] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    deps.append(os.path.join(ROOT, "include", "gbp.h"))
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc(), "-c", path, "-o", obj, *_flags(src)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    if r.stderr.strip() and os.environ.get("GBP_PTXAS_VERBOSE"):
        sys.stderr.write(r.stderr)
    return obj


def build(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if force:
        for f in os.listdir(BUILD):
            os.unlink(os.path.join(BUILD, f))
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, srcs))
    if os.path.exists(LIB) and not force and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs):
        return LIB
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared", "-o", tmp, *objs, *ARCH, "-cudart", "static", "-Xlinker", "-z,defs", "-lrt",
           "-lpthread", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
