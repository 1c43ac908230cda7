"""The cluster LDL^T solve of the reduced camera system, called directly
(tests/cpp/chol_probe.cu) on matrices laid out like the solver's S: results
against numpy from 1 to 384 unknowns (every cluster size and backward-solve
staging depth), the failure path of an indefinite system (LinearSolverEigen
reports failure and leaves x untouched, linear_solver_eigen.h:118-126), and
the bounded waits: a flag that no worker releases must end in a failed solve
within seconds, with the context still usable afterwards."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SENTINEL = 12345.0


@pytest.fixture(scope="module")
def probe(tmp_path_factory, gpu):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out = str(tmp_path_factory.mktemp("probe") / "libchol_probe.so")
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
           "-shared", "-I", os.path.join(ROOT, "mcvslam_gb300", "csrc"),
           os.path.join(ROOT, "tests", "cpp", "chol_probe.cu"), "-o", out]
    subprocess.run(cmd, check=True)
    L = ctypes.CDLL(out)
    dp = ctypes.POINTER(ctypes.c_double)
    L.chol_probe_solve.argtypes = [dp, ctypes.c_int, ctypes.c_int, dp, ctypes.c_int,
                                   ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_float)]
    L.chol_probe_solve.restype = ctypes.c_int
    return L


def _solve(L, A, b, hold=False):
    n = A.shape[0]
    ld = 32 * ((n + 31) // 32)
    S = np.zeros((ld + 32, ld))
    S[:n, :n] = A
    for i in range(n, ld):
        S[i, i] = 1.0
    S[ld, :n] = b
    x = np.full(ld, SENTINEL)
    ok = ctypes.c_int(-1)
    ms = ctypes.c_float(0.0)
    dp = ctypes.POINTER(ctypes.c_double)
    rc = L.chol_probe_solve(S.ctypes.data_as(dp), n, ld, x.ctypes.data_as(dp), int(hold), ctypes.byref(ok),
                            ctypes.byref(ms))
    return rc, x[:n], ok.value, ms.value


def _spd(n, seed):
    rng = np.random.default_rng(seed)
    M = rng.standard_normal((n, n))
    return M @ M.T + n * np.eye(n), rng.standard_normal(n)


@pytest.mark.parametrize("n", [1, 5, 16, 17, 48, 72, 100, 168, 240, 300, 384])
def test_cluster_solve_matches_numpy(probe, n):
    A, b = _spd(n, 1000 + n)
    rc, x, ok, _ = _solve(probe, A, b)
    assert rc == 0 and ok == 1
    ref = np.linalg.solve(A, b)
    assert np.abs(x - ref).max() <= 1e-12 * np.abs(ref).max()


def test_indefinite_system_fails_and_leaves_x(probe):
    A, b = _spd(168, 7)
    A[100, 100] = -A[100, 100]
    rc, x, ok, _ = _solve(probe, A, b)
    assert rc == 0 and ok == 0
    assert np.all(x == SENTINEL)


@pytest.mark.parametrize("hold", [1, 2], ids=["rhs_panel_flag", "inverse_flag"])
def test_wait_that_runs_out_ends_in_a_failed_solve(probe, hold):
    """A flag the workers leave unreleased (the first right-hand-side panel's,
    or the first backward-solve inverse's): the waits on it give up after
    their 1 s limit, the solve reports failure, and the context stays
    usable."""
    A, b = _spd(168, 8)
    rc, _, ok, ms = _solve(probe, A, b, hold=hold)
    assert rc == 0 and ok == 0
    assert ms < 20000.0
    # the context is still usable: the same system solves normally
    rc, x, ok, _ = _solve(probe, A, b)
    assert rc == 0 and ok == 1
    ref = np.linalg.solve(A, b)
    assert np.abs(x - ref).max() <= 1e-12 * np.abs(ref).max()
