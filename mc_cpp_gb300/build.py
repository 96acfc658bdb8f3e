"""Builds libmcgpu.so in-tree (mc_cpp_gb300/_lib/) for sm_103a, without CMake.

    python -m mc_cpp_gb300.build            # or __graft_entry__.build()

Translation units are compiled in parallel; objects go to mc_cpp_gb300/_build/ (git-ignored).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libmcgpu.so")
SHIM_SRC = os.path.join(HERE, "shim", "charmmene_gpu.cpp")
SHIM = os.path.join(LIBDIR, "libcharmmene_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nv = shutil.which("nvcc")
    if nv:
        return os.path.dirname(os.path.dirname(nv))
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _sources():
    return sorted(f for f in os.listdir(SRC) if f.endswith((".cu", ".cpp")))


def _compile(src: str, cuda: str) -> str:
    path = os.path.join(SRC, src)
    obj = os.path.join(BUILD, src + ".o")
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + SRC]
    if src.endswith(".cu"):
        # -ftz=true: FP32 subnormals flush to zero (no pair term, displacement or partial sum is
        # subnormal); the FP64 plain path is unaffected
        cmd = [os.path.join(cuda, "bin", "nvcc")] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-ftz=true", "-Xcompiler", "-fPIC",
                                                             "-diag-suppress", "1444", "-c", path, "-o", obj] + inc
    else:
        cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-c", path, "-o", obj,
               "-I" + os.path.join(cuda, "include")] + inc
    deps = [path] + [os.path.join(SRC, h) for h in os.listdir(SRC) if h.endswith((".hpp", ".cuh"))] + \
           [os.path.join(ROOT, "include", "mcg.h")]
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return obj


def build(verbose: bool = False) -> str:
    cuda = _cuda_home()
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, cuda), srcs))
    if not (os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs)):
        cmd = [os.path.join(cuda, "bin", "nvcc")] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + \
              ["-lcudart_static", "-lrt", "-lpthread", "-ldl"]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s" % (" ".join(cmd), r.stdout))
        os.replace(LIB + ".tmp", LIB)
    _build_shim()
    if verbose:
        print("built", LIB)
    return LIB


def _build_shim() -> str:
    """libcharmmene_gpu.so: the reference's Fortran/C energy interface on top of libmcgpu.so."""
    deps = [SHIM_SRC, LIB, os.path.join(ROOT, "include", "charmmene_gpu.h"), os.path.join(ROOT, "include", "mcg.h")]
    if os.path.exists(SHIM) and os.path.getmtime(SHIM) >= max(os.path.getmtime(d) for d in deps):
        return SHIM
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-Wall", SHIM_SRC, "-I" + os.path.join(ROOT, "include"),
           "-L" + LIBDIR, "-lmcgpu", "-Wl,-rpath,$ORIGIN", "-o", SHIM + ".tmp"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("shim build failed: %s\n%s" % (" ".join(cmd), r.stdout))
    os.replace(SHIM + ".tmp", SHIM)
    return SHIM


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
