"""Builds libgraspgpu.so (CUDA, sm_103a) and libgraspangular.so (host C++,
the T/V list producer) in-tree.

Run ``python -m grasp_gb300.build`` or call :func:`build`. Objects go to
``grasp_gb300/_build/``; translation units compile in parallel.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
INC = os.path.join(os.path.dirname(HERE), "include")

GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = GENCODE + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INC]
# files whose FP64 arithmetic restates the reference step by step: no
# contraction of a*b + c into one fused rounding
NO_FMAD = {"radial.cu", "setham.cu", "spmv.cu", "davidson.cu", "breit.cu", "setcof.cu"}  # exact FP64 sums; error-free double-float steps
CU_SOURCES = ["ctx.cu", "radial.cu", "setham.cu", "spmv.cu", "davidson.cu", "bdvd.cu", "hostmat.cu", "breit.cu", "setcof.cu"]
CPP_SOURCES = ["hosteig.cpp"]
ANGULAR_SOURCES = ["angular.cpp"]

LIB_GPU = os.path.join(OUT, "libgraspgpu.so")
LIB_ANGULAR = os.path.join(OUT, "libgraspangular.so")


def _nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgraspgpu")
    return p


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INC, f) for f in os.listdir(INC) if f.endswith(".h")]
    return hs


def build(force: bool = False, verbose: bool = False, ptxas_verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers()
    jobs = []
    objs = []
    for f in CU_SOURCES:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT, f + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            flags = list(NVCC_FLAGS)
            if f in NO_FMAD:
                flags.append("-fmad=false")
            if ptxas_verbose:
                flags += ["-Xptxas", "-v"]
            jobs.append([nvcc] + flags + ["-c", src, "-o", obj])
    for f in CPP_SOURCES:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT, f + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", "-I" + INC, "-c", src, "-o", obj])
    relink = bool(jobs)
    ang_srcs = [os.path.join(CSRC, f) for f in ANGULAR_SOURCES]
    if force or _stale(LIB_ANGULAR, ang_srcs + hdrs):
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I" + INC, "-o", LIB_ANGULAR] + ang_srcs +
                    ["-lpthread"])
    logs = []
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            logs.append(out)
    if force or relink or not os.path.exists(LIB_GPU):
        _run([nvcc] + GENCODE + ["-shared", "-o", LIB_GPU] + objs)
    if verbose:
        for l in logs:
            if l.strip():
                print(l)
    return LIB_GPU


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_verbose="--ptxas" in sys.argv)
    print(LIB_GPU)
