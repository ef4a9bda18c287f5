"""Build the native libraries of louvain-gb300 in-tree.

Products (written to ``lib/`` beside this file; git-ignored):

* ``liblouvain_gb300.so`` — the GB300 Louvain library: hand-written sm_103a CUDA
  kernels behind the C-ABI declared in ``include/louvain_gb300.h``.
* ``liblvg_graphgen.so`` — host-only seeded graph and batch generators and
  the SNAP temporal reader (``include/louvain_gb300_graphgen.h``); no CUDA
  dependency.
* ``louvain_gb300_experiment`` — the reference's experiment driver (main.cxx)
  over the two libraries: same command line, same log lines.

Every CUDA translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, then linked with
``nvcc -shared``. Objects whose source and headers are unchanged are reused.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(HERE, "lib")
OBJ = os.path.join(LIB, "obj")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
              "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC]
CXX_FLAGS = ["-std=c++17", "-O3", "-fPIC", "-fopenmp", "-I", INCLUDE]

CUDA_LIB = os.path.join(LIB, "liblouvain_gb300.so")
GEN_LIB = os.path.join(LIB, "liblvg_graphgen.so")
EXPERIMENT = os.path.join(LIB, "louvain_gb300_experiment")


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the CUDA 13 toolkit is required to build liblouvain_gb300.so")
    return cand


def _headers() -> list[str]:
    hs = []
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            if f.endswith((".cuh", ".h", ".hxx", ".hpp")):
                hs.append(os.path.join(d, f))
    return hs


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}):\n{' '.join(cmd)}\n{r.stdout}")
    if verbose and r.stdout.strip():
        print(r.stdout, flush=True)


def build_graphgen(verbose: bool = False) -> str:
    os.makedirs(LIB, exist_ok=True)
    src = os.path.join(CSRC, "lvg_graphgen.cpp")
    if _stale(GEN_LIB, [src] + _headers()):
        _run(["g++", *CXX_FLAGS, "-shared", src, "-o", GEN_LIB], verbose)
    return GEN_LIB


def build_cuda(verbose: bool = False, extra_flags: list[str] | None = None) -> str:
    os.makedirs(OBJ, exist_ok=True)
    nvcc = _nvcc()
    srcs = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))
    hdrs = _headers()
    flags = NVCC_FLAGS + list(extra_flags or [])
    jobs = []
    objs = []
    for s in srcs:
        o = os.path.join(OBJ, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if _stale(o, [s] + hdrs + [os.path.abspath(__file__)]):
            jobs.append([nvcc, *ARCH, *flags, "-c", s, "-o", o])
    if jobs:
        with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
            list(ex.map(lambda c: _run(c, verbose), jobs))
    if jobs or _stale(CUDA_LIB, objs):
        _run([nvcc, *ARCH, "-shared", *objs, "-o", CUDA_LIB, "-lcudart"], verbose)
    return CUDA_LIB


def build_experiment(verbose: bool = False) -> str:
    src = os.path.join(CSRC, "lvg_experiment.cpp")
    if _stale(EXPERIMENT, [src, CUDA_LIB, GEN_LIB] + _headers()):
        _run([_nvcc(), "-std=c++17", "-O2", "-I", INCLUDE, src, "-o", EXPERIMENT, "-L", LIB, "-llouvain_gb300",
              "-llvg_graphgen", "-lcudart", "-Xlinker", "-rpath,$ORIGIN"], verbose)
    return EXPERIMENT


def build(verbose: bool = False) -> None:
    build_graphgen(verbose)
    build_cuda(verbose)
    build_experiment(verbose)


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
