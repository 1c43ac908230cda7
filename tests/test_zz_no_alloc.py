"""The allocation-free robust-cost entry point, checked against the solver.

Callers that cannot allocate device memory -- a tracking thread with a hard
per-frame deadline, where cudaMalloc/cudaFree may wait for the whole device, or
an application whose own pool owns all device memory -- use
mcba_robust_cost_noalloc, which keeps its scratch in a fixed static device
array.  Its sum must equal the initial robust chi2 that mcba_optimize computes
with library-allocated scratch, on two calls in a row (the shared array keeps
the previous call's contents and must not leak them into the next result).
This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

from mcvslam_gb300 import _native as N
from mcvslam_gb300 import ba, synth
from oracle import oracle

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def _edge_arrays(pr, qt):
    ext = np.stack([oracle.mat44f_to_qt(pr.cam_Tcb[c]) for c in range(pr.n_cams)])
    return {
        "pose": np.ascontiguousarray(qt[pr.edge_pose]),
        "ext": np.ascontiguousarray(ext[pr.edge_cam]),
        "X": np.ascontiguousarray(pr.point_Xw[pr.edge_point].astype(np.float64)),
        "K": np.ascontiguousarray(pr.cam_K[pr.edge_cam].astype(np.float64)),
        "obs": np.ascontiguousarray(pr.edge_obs[:, :2].astype(np.float64)),
        "info": pr.edge_info.astype(np.float64),
        "delta": pr.edge_delta.astype(np.float64),
        "robust": pr.edge_robust.astype(np.uint8),
    }


def test_noalloc_cost_matches_the_solver_twice(gpu):
    torch = pytest.importorskip("torch")
    pr = synth.config(1)
    with ba.Solver() as s:
        s.load(pr)
        ref = s.optimize(0)["initial_chi2"]
        qt, _ = s.state()
    host = _edge_arrays(pr, qt)
    dev = {k: torch.from_numpy(v).cuda() for k, v in host.items()}
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    L = N.lib()
    for call in range(2):
        r = L.mcba_robust_cost_noalloc(pr.n_edges, dev["pose"].data_ptr(), dev["ext"].data_ptr(),
                                       dev["X"].data_ptr(), dev["K"].data_ptr(), dev["obs"].data_ptr(),
                                       dev["info"].data_ptr(), dev["delta"].data_ptr(), dev["robust"].data_ptr(),
                                       out.data_ptr(), None)
        assert r == N.MCBA_OK
        torch.cuda.synchronize()
        cost = float(out.item())
        assert abs(cost - ref) <= RTOL * ref, (call, cost, ref)
        out.fill_(-1.0)


def test_noalloc_rejects_batches_above_its_scratch(gpu):
    torch = pytest.importorskip("torch")
    one = torch.zeros(8, dtype=torch.float64, device="cuda")
    L = N.lib()
    p = one.data_ptr()
    r = L.mcba_robust_cost_noalloc(N.NOALLOC_MAX_EDGES + 1, p, p, p, p, p, None, None, None, p, None)
    assert r == N.MCBA_ERR_TOO_LARGE
