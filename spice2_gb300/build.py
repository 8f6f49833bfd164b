"""Builds libspice_gb300.so (the CUDA engine behind include/spice_gb300.h) in-tree.

nvcc compiles every translation unit for sm_103a only (one -gencode, -lineinfo), in parallel, and
links them into spice2_gb300/libspice_gb300.so.  Device code is built with -fmad=false and host
code with -ffp-contract=off so that every floating-point operation is a single IEEE
round-to-nearest operation, as the parity with the reference requires.
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
LIB = os.path.join(HERE, "libspice_gb300.so")

SOURCES = ["rng_host.cpp", "gen.cu", "step.cu", "net.cu", "noalloc.cu", "batch.cu", "adjoint.cu", "pull.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    p = os.path.join(cuda, "bin", "nvcc")
    return p if os.path.exists(p) else (shutil.which("nvcc") or "nvcc")


def common_flags() -> list[str]:
    return ["-std=c++17", "-O3", "-lineinfo", "-fmad=false", "--expt-relaxed-constexpr",
            "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-I" + CSRC, "-I" + os.path.join(ROOT, "include")]


def _compile(src: str) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    srcp = os.path.join(CSRC, src)
    deps = [srcp] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    deps.append(os.path.join(ROOT, "include", "spice_gb300.h"))
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc()] + ARCH + common_flags() + ["-c", srcp, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc()] + ARCH + common_flags() + ["-x", "cu", "-c", srcp, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    if os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(o) for o in objs):
        return LIB
    cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
