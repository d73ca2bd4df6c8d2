"""Build the CUDA library ``libmclum.so`` in-tree with nvcc (sm_103a only).

``build()`` compiles every ``csrc/*.cu`` translation unit in parallel and links
them into ``mcluminescence_gb300/lib/libmclum.so``; it skips the work when the
library is newer than every source and header.  No CMake, no torch extension
machinery: the library exposes a plain C ABI (``include/mclum.h``) that
``_lib.py`` loads with ctypes.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(REPO, "include")
OBJDIR = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libmclum.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC]
# Every kernel whose results are compared bit for bit keeps each multiply and
# add rounded on its own (no contraction into FMA).  The fused surrogate
# network is compared within a tolerance, so it lets the compiler contract.
CONTRACT = {"mlp_fused.cu"}


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found (set NVCC or put the CUDA toolkit on PATH)")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return _sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h")) \
        + [os.path.abspath(__file__)]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def _compile(nvcc, src, extra, verbose):
    obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
    fmad = "-fmad=true" if os.path.basename(src) in CONTRACT else "-fmad=false"
    cmd = [nvcc] + NVCC_FLAGS + [fmad] + list(extra) + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        print(r.stdout + r.stderr)
    return obj


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> str:
    """Compile and link the library; returns its path."""
    if not force and not extra_flags and up_to_date():
        return LIB
    nvcc = nvcc_path()
    os.makedirs(OBJDIR, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=max(1, min(os.cpu_count() or 8, len(srcs)))) as ex:
        objs = list(ex.map(lambda s: _compile(nvcc, s, extra_flags, verbose), srcs))
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True,
                extra_flags=["-Xptxas", "-v"] if "--ptxas" in sys.argv else ()))
