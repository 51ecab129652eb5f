"""Builds libtracer_gpu.so in-tree with nvcc for sm_103a.

Translation units compile in parallel; the result is linked next to this file
(tracer_code_gb300/libtracer_gpu.so).  Device code uses --fmad=false (the
kernels that must equal the CPU restatement bit for bit rely on it; fused
multiply-adds are written explicitly where wanted) and host code uses
-ffp-contract=off for the same reason on aarch64 hosts.
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
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libtracer_gpu.so")

SOURCES = ["k_mg.cu", "k_visit.cu", "k_sweepblk.cu", "k_mixed.cu", "k_conv.cu", "k_nn.cu", "tc_nn_api.cu", "k_field.cu", "k_tracer.cu", "k_noalloc.cu", "k_subcycle.cu", "k_accel.cu", "k_loop.cu", "tc_api.cu", "tc_setup.cpp", "tc_restart.cpp", "tc_format.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def common_flags() -> list[str]:
    return ARCH + [
        "-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off,-fopenmp",
        "-I", INCLUDE, "-I", CSRC,
    ]


def _deps(src: str) -> list[str]:
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    pub = [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return [os.path.join(CSRC, src)] + pub + hdrs


def _compile(src: str, force: bool) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    if not force and os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in _deps(src)):
        return obj
    cmd = [nvcc_path(), "-c", os.path.join(CSRC, src), "-o", obj] + common_flags()
    if src.endswith(".cpp"):
        cmd += ["-x", "c++"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, force), SOURCES))
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc_path(), "-shared", "-o", LIB] + objs + ARCH + ["-Xcompiler", "-fopenmp", "-lgomp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
