"""Builds libxpbd_gb300.so in-tree for sm_103a.

CUDA sources are compiled by nvcc with --fmad=false (no implicit fused
multiply-add: the kernels must reproduce the reference's arithmetic order),
host C++ by g++ with -ffp-contract=off, both in parallel, then linked by nvcc.
A hash of the sources and flags decides whether anything needs rebuilding.
"""
from __future__ import annotations

import hashlib
import os
import platform
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(os.path.dirname(ROOT), "include")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libxpbd_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-I" + INCLUDE]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function", "-I" + INCLUDE]


def _cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def _sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    hdr = sorted(f for f in os.listdir(CSRC) if f.endswith((".h", ".cuh")))
    return cu, cpp, hdr


def _digest(cu, cpp, hdr) -> str:
    h = hashlib.sha256()
    h.update(" ".join(ARCH + NVCC_FLAGS + CXX_FLAGS + [platform.machine()]).encode())
    for f in cu + cpp + hdr:
        with open(os.path.join(CSRC, f), "rb") as fh:
            h.update(f.encode() + fh.read())
    with open(os.path.join(INCLUDE, "xpbd.h"), "rb") as fh:
        h.update(fh.read())
    return h.hexdigest()


def build_library(force: bool = False, verbose: bool = False, jobs: int | None = None) -> str:
    cu, cpp, hdr = _sources()
    digest = _digest(cu, cpp, hdr)
    stamp = os.path.join(BUILD, "stamp")
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as fh:
            if fh.read().strip() == digest:
                return LIB
    os.makedirs(BUILD, exist_ok=True)
    home = _cuda_home()
    nvcc = os.path.join(home, "bin", "nvcc")
    cuda_inc = os.path.join(home, "include")
    cmds = []
    for f in cu:
        obj = os.path.join(BUILD, f + ".o")
        cmds.append([nvcc, *ARCH, *NVCC_FLAGS, "-c", os.path.join(CSRC, f), "-o", obj])
    for f in cpp:
        obj = os.path.join(BUILD, f + ".o")
        cmds.append([os.environ.get("CXX", "g++"), *CXX_FLAGS, "-I" + cuda_inc, "-c", os.path.join(CSRC, f), "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        for out in ex.map(run, cmds):
            if verbose and out:
                print(out)
    objs = [os.path.join(BUILD, f + ".o") for f in cu + cpp]
    tmp = LIB + ".tmp"
    run([nvcc, *ARCH, "-shared", "-Xcompiler", "-fPIC", *objs, "-o", tmp])
    os.replace(tmp, LIB)
    with open(stamp, "w") as fh:
        fh.write(digest)
    return LIB


if __name__ == "__main__":
    import sys
    print(build_library(force="--force" in sys.argv, verbose=True))
