"""Build the CUDA library in-tree: pcaone_gb300/lib/libpcaone_gb300.so.

Each translation unit is compiled separately (in parallel) for sm_103a and
linked with nvcc; the host RNG file is compiled by g++ with FP contraction
into FMAs, as the reference's own build does.  No torch or CMake involvement.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIBNAME = "libpcaone_gb300.so"
LIBPATH = os.path.join(LIBDIR, LIBNAME)

CU_SOURCES = ["bed.cu", "prod_simt.cu", "prod_tc.cu", "dense64.cu", "util.cu", "halko.cu", "noalloc.cu", "mlp.cu", "project.cu"]
CPP_SOURCES = ["rng.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# The host random streams (rng.cpp) contract the polar method's arithmetic into
# fused multiply-adds, as the reference's own build (-march=native / -mcpu=native)
# does on both host types, so that the drawn test matrix is the reference's bit
# for bit: FMA is part of the Arm base ISA, on x86-64 it is enabled by -mfma.
RNG_FLAGS = ["-ffp-contract=fast"] + (["-mfma"] if platform.machine() in ("x86_64", "AMD64") else [])


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _stale(obj: str, srcs) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(s) > t for s in srcs)


def build(verbose: bool = False, force: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(OBJDIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "pcaone_gpu.h"))
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJDIR, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmd = [nvcc(), *ARCH, "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler",
                   "-ffp-contract=off", "--expt-relaxed-constexpr", "-c", s, "-o", o]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJDIR, src + ".o")
        objs.append(o)
        if force or _stale(o, [s]):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", *RNG_FLAGS, "-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for out in ex.map(_run, jobs):
                if verbose and out.strip():
                    print(out)
    if force or jobs or not os.path.exists(LIBPATH):
        tmp = LIBPATH + f".tmp{os.getpid()}"
        _run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"])
        os.replace(tmp, LIBPATH)
    return LIBPATH


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv, ptxas_info="--ptxas" in sys.argv))
