"""Host-side layout checks of the cluster LDL^T (tests/cpp/chol_layout.cu):
alignment of the workspace tiles and push targets, the flag array's place in
the chain CTA's shared memory, the workspace size and the shared memory
total, for 1..384 unknowns and every cluster size.  Compiled for sm_103a and
run on the host; no device call."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cluster_solve_layout(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "chol_layout")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O1",
                    "-I", os.path.join(ROOT, "mcvslam_gb300", "csrc"), "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "chol_layout.cu"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout[-2000:]
    assert "layout ok" in out.stdout
