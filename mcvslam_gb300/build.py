"""Build recipe for libmcba.so (sm_103a only).

Every translation unit is compiled in parallel with nvcc and linked into
mcvslam_gb300/_build/libmcba.so (git-ignored, rebuilt on each host since the
library is architecture specific).  No torch, no cmake.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(OUT, "libmcba.so")

SOURCES = ["mcba_api.cpp", "mcba_solver.cu", "mcba_chol.cu", "mcba_chol_tiled.cu", "mcba_batch.cu", "mcba_reproj.cu", "mcba_noalloc.cu", "mcba_compile.cu", "mcba_match.cu", "mcba_project.cu", "mcba_stereo.cu", "mcba_window.cu", "mcba_peak.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    files.append(os.path.abspath(__file__))
    return files


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(f) > t for f in _deps())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    nv = nvcc()
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC]
    procs = []
    objs = []
    for src in SOURCES:
        path = os.path.join(CSRC, src)
        if not os.path.exists(path):
            continue
        obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
        objs.append(obj)
        if src.endswith(".cu"):
            cmd = [nv, *ARCH, "-lineinfo", *common, "-c", path, "-o", obj]
        else:
            cmd = [nv, *common, "-x", "c++", "-c", path, "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((src, subprocess.Popen(cmd)))
    for src, p in procs:
        if p.wait() != 0:
            raise RuntimeError(f"nvcc failed on {src}")
    tmp = LIB + ".tmp"
    cmd = [nv, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-lpthread", "-ldl"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    if subprocess.call(cmd) != 0:
        raise RuntimeError("link of libmcba.so failed")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
