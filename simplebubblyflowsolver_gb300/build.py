"""Build libsbfs_gb300.so in-tree: hand-written CUDA for sm_103a plus host C++.

    python -m simplebubblyflowsolver_gb300.build

Each translation unit is compiled in parallel, then linked with nvcc.  The
only target is sm_103a (GB300); there is no other architecture and no
fallback.
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
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libsbfs_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["sbfs_kernels.cu", "sbfs_api.cu", "sbfs_noalloc.cu", "sbfs_mlp.cu"]
CXX_SOURCES = ["sbfs_npyio.cpp"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the library")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _sources_newer(target: str) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(p) > t for p in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _sources_newer(LIB):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INCLUDE]
    jobs = []
    for src in CUDA_SOURCES:
        obj = os.path.join(BUILD, src + ".o")
        jobs.append([nv, *ARCH, "-lineinfo", *common, "-c", os.path.join(CSRC, src), "-o", obj])
    for src in CXX_SOURCES:
        obj = os.path.join(BUILD, src + ".o")
        jobs.append([nv, *common, "-x", "c++", "-c", os.path.join(CSRC, src), "-o", obj])
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    objs = [os.path.join(BUILD, s + ".o") for s in CUDA_SOURCES + CXX_SOURCES]
    tmp = LIB + ".tmp"
    _run([nv, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
