"""Builds ug_gb300/lib/libug_gb300.so in tree.

CUDA sources are compiled for GB300 only (-gencode arch=compute_103a,code=sm_103a),
host C++ with g++; the objects are linked against the CUDA runtime.  Objects
are rebuilt only when a source or header is newer.  Runs on x86_64 and on the
aarch64 GPU hosts alike (no architecture-specific host flags).

    python -m ug_gb300.build        # or: python ug_gb300/build.py
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libug_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

GENCODE = "-gencode=arch=compute_103a,code=sm_103a"


def cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nv = shutil.which("nvcc")
    if nv:
        return os.path.dirname(os.path.dirname(nv))
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _deps():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + _deps() + [os.path.abspath(__file__)])


def build(verbose: bool = False) -> str:
    cuda = cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    jobs = []
    objs = []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, src):
            jobs.append([nvcc, GENCODE, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                         "-Xptxas", "-warn-spills", "-I" + INCLUDE, "-c", src, "-o", obj])
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cpp"))):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, src):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-variable",
                         "-I" + os.path.join(cuda, "include"), "-I" + INCLUDE, "-c", src, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        for err in ex.map(run, jobs):
            if verbose and err.strip():
                print(err)
    if jobs or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        libdir = os.path.join(cuda, "lib64")
        if not os.path.isdir(libdir):
            libdir = os.path.join(cuda, "lib")
        tmp = LIB + ".tmp"
        run(["g++", "-shared", "-o", tmp] + objs + ["-L" + libdir, "-lcudart", "-Wl,-rpath," + libdir, "-lpthread"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
