"""Builds the solver's native code in-tree, for sm_103a only.

Outputs (git-ignored, rebuilt wherever the code runs):
  pps/libpps_gb.so   the C-ABI library (kernels, engine, compiler, queries)
  pps/gpu_pfflop     the command-line driver (reference CLI protocol)

Objects go to _build/; translation units compile in parallel and are only
rebuilt when a source or header is newer than the object.

    python cuda-poker-solver_gb300/build_ext.py [--force] [--verbose]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "pps", "libpps_gb.so")
CLI = os.path.join(PKG, "pps", "gpu_pfflop")
INCLUDES = ["-I", os.path.join(REPO, "include", "pps"), "-I", os.path.join(REPO, "include"),
            "-I", CSRC]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
LIB_SOURCES = ["cards.cpp", "bet_tree.cpp", "compiler.cpp", "layout.cpp", "solver.cpp",
               "capi.cpp", "gpu_cfr.cpp", "tune.cpp", "engine.cu", "rowcodec.cu", "noalloc.cu", "forest.cu", "batch.cpp"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _headers_mtime():
    m = 0.0
    for d in (CSRC, os.path.join(REPO, "include"), os.path.join(REPO, "include", "pps")):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh")):
                m = max(m, os.path.getmtime(os.path.join(d, f)))
    return m


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("build failed:\n%s\n%s%s" % (" ".join(cmd), p.stdout, p.stderr))
    return p.stdout + p.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    nvcc = _nvcc()
    hdr = _headers_mtime()
    jobs = []
    objs = []
    for src in LIB_SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(OBJ, src + ".o")
        objs.append(obj)
        stale = force or not os.path.exists(obj) or \
            os.path.getmtime(obj) < max(os.path.getmtime(path), hdr)
        if not stale:
            continue
        flags = ["-std=c++17", "-O3", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall"] + INCLUDES
        if src.endswith(".cu"):
            flags += ARCH + ["-lineinfo"]
        jobs.append([nvcc] + flags + ["-c", path, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        list(ex.map(lambda c: _run(c, verbose), jobs))
    if jobs or force or not os.path.exists(LIB):
        _run([nvcc, "-shared"] + ARCH + ["-o", LIB] + objs + ["-lcudart"], verbose)
    cli_src = os.path.join(CSRC, "gpu_pfflop.cpp")
    if force or not os.path.exists(CLI) or os.path.getmtime(CLI) < max(
            os.path.getmtime(LIB), os.path.getmtime(cli_src)):
        _run(["g++", "-std=c++17", "-O2"] + INCLUDES + [cli_src, "-o", CLI,
              "-L" + os.path.dirname(LIB), "-lpps_gb", "-Wl,-rpath,$ORIGIN"], verbose)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="--verbose" in sys.argv))
