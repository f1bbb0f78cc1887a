"""In-tree build of libtennet_cuda.so for sm_103a (GB300).

Compiles every CUDA and C++ translation unit of ``csrc/`` in parallel with nvcc / g++ and
links one shared library into ``lib/``.  No cmake, no torch extension machinery.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libtennet_cuda.so")
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"]
CXX_FLAGS = ["-O2", "-fPIC", "-std=c++17", "-Wall", "-Wno-unused-function",
             f"-I{CUDA_HOME}/include"]


def _sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    return cu, cpp


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    """Build (if stale) and return the path of libtennet_cuda.so."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    cu, cpp = _sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".h")]
    headers.append(os.path.join(INCLUDE, "tennet.h"))
    jobs = []
    objs = []
    for f in cu:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([NVCC, *ARCH, *NVCC_FLAGS, f"-I{INCLUDE}", "-c", src, "-o", obj])
    cxx = shutil.which("g++") or "g++"
    for f in cpp:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([cxx, *CXX_FLAGS, f"-I{INCLUDE}", "-c", src, "-o", obj])
    logs = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=max(2, min(len(jobs), os.cpu_count() or 4))) as ex:
            for out in ex.map(_run, jobs):
                logs.append(out)
    if force or jobs or _stale(LIB, objs):
        logs.append(_run([NVCC, *ARCH, "-shared", "-o", LIB, *objs, "-lpthread"]))
    if verbose:
        for line in logs:
            if line.strip():
                print(line)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
