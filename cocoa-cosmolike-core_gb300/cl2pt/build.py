"""Build libcl2pt.so in-tree with nvcc for sm_103a (GB300).

Translation units compile in parallel; the shared library lands next to
this file.  No cmake, no torch extension machinery.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INC = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(HERE, "libcl2pt.so")
LEGACY = os.path.join(HERE, "libcl2pt_legacy.so")
LEGACY_SRC = os.path.join(CSRC, "legacy", "legacy.cpp")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code without floating-point contraction, so that plan-time tables
# (filters, node flags) round the same on x86-64 and aarch64
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", f"-I{INC}",
         f"-I{CSRC}"]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libcl2pt")
    return p


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _newer(dst: str, srcs) -> bool:
    if not os.path.exists(dst):
        return False
    t = os.path.getmtime(dst)
    return all(os.path.getmtime(s) <= t for s in srcs)


def headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INC, f) for f in os.listdir(INC) if f.endswith(".h")]
    return hs


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    hs = headers() + [os.path.abspath(__file__)]  # a change of flags rebuilds
    jobs = []
    objs = []
    for src in sources():
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or not _newer(obj, [src] + hs):
            jobs.append([cc, *ARCH, *FLAGS, "-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
            futs = [ex.submit(subprocess.run, j, capture_output=True, text=True) for j in jobs]
            for j, f in zip(jobs, futs):
                r = f.result()
                if verbose or r.returncode:
                    print(" ".join(j))
                    print(r.stdout, r.stderr)
                if r.returncode:
                    raise RuntimeError(f"nvcc failed on {j[-3]}")
    if force or jobs or not _newer(LIB, objs):
        cmd = [cc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            print(r.stdout, r.stderr)
            raise RuntimeError("link of libcl2pt.so failed")
    build_legacy(force)
    return LIB


def build_legacy(force: bool = False) -> str:
    """libcl2pt_legacy.so: the reference-named entry points (host C++ over
    libcl2pt.so, found next to it at run time)."""
    if not force and _newer(LEGACY, [LEGACY_SRC, LIB] + headers()):
        return LEGACY
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-O2", "-std=c++17", "-fPIC", "-shared", f"-I{INC}", LEGACY_SRC, "-o", LEGACY,
           f"-L{HERE}", "-lcl2pt", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        print(" ".join(cmd))
        print(r.stdout, r.stderr)
        raise RuntimeError("build of libcl2pt_legacy.so failed")
    return LEGACY


if __name__ == "__main__":
    print(build(verbose=True))
