"""The header-only C++ BAoptimizer shim compiles against libmcba.so and its
host-side bookkeeping works (no GPU needed)."""
import os
import shutil
import subprocess

import pytest

from mcvslam_gb300 import _native as N

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_shim_builds_and_runs_host_side(tmp_path):
    if not shutil.which("g++"):
        pytest.skip("no g++")
    N.lib()  # builds libmcba.so if needed
    libdir = os.path.dirname(N.LIB_PATH)
    exe = str(tmp_path / "shim_host")
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "shim_host.cpp"), "-L", libdir, "-lmcba",
           "-Wl,-rpath," + libdir, "-o", exe]
    subprocess.run(cmd, check=True)
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, (out.returncode, out.stdout, out.stderr)
    assert "shim ok" in out.stdout
