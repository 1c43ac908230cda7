"""Build recipe for the CPU oracle (test infrastructure, not product code).

Compiles oracle/g2o_oracle.cpp, matcher_oracle.cpp and window_oracle.cpp twice into
oracle/_build/:
  liboracle.so      serial restatement (the reference's g2o is built with
                    OpenMP off, ThirdParty/g2o/CMakeLists.txt:139-149)
  liboracle_omp.so  the same source with OpenMP, for the multi-core baseline
Portable flags only (the library is rebuilt on each host architecture);
floating-point contraction is off so x86 and Arm builds agree bit for bit.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
SRC = os.path.join(HERE, "g2o_oracle.cpp")
SRC_MATCH = os.path.join(HERE, "matcher_oracle.cpp")
SRC_WINDOW = os.path.join(HERE, "window_oracle.cpp")
HDR = os.path.join(HERE, "g2o_oracle.h")

TARGETS = {
    "liboracle.so": [],
    "liboracle_omp.so": ["-fopenmp"],
}


def _stale(out: str) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in (SRC, SRC_MATCH, SRC_WINDOW, HDR, __file__))


def build(force: bool = False, verbose: bool = False) -> dict:
    os.makedirs(OUT, exist_ok=True)
    paths = {}
    procs = []
    for name, extra in TARGETS.items():
        out = os.path.join(OUT, name)
        paths[name] = out
        if force or _stale(out):
            cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
                   "-Wall", "-Wno-unknown-pragmas", *extra, "-o", out + ".tmp", SRC, SRC_MATCH, SRC_WINDOW]
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
            procs.append((out, subprocess.Popen(cmd)))
    for out, p in procs:
        if p.wait() != 0:
            raise RuntimeError(f"oracle build failed: {out}")
        os.replace(out + ".tmp", out)
    return paths


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
