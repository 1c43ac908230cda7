"""Reprojection residual as a torch.autograd.Function over the CUDA kernels.

1M random edges (rotations uniform on SO(3), translations N(0, 5 m), the
baseline rig's extrinsics, points at depth U(1, 50) m), FP64 and FP32:
* forward residual vs an FP64 NumPy evaluation of the same formula;
* backward (J^T g) vs FP64 central finite differences (h = 1e-6) through the
  same forward kernel;
* J_pose and J_X vs the oracle's restatement of linearizeOplus
  (include/OptimizeTypes.hpp:94-113) on the same edges.
"""
import numpy as np
import pytest

from mcvslam_gb300 import synth
from oracle import oracle

pytestmark = pytest.mark.gpu

N_EDGES = 1_000_000


def _q1(R):
    tr = np.trace(R)
    if tr > 0:
        s = np.sqrt(tr + 1.0)
        w = 0.5 * s
        s = 0.5 / s
        q = np.array([(R[2, 1] - R[1, 2]) * s, (R[0, 2] - R[2, 0]) * s, (R[1, 0] - R[0, 1]) * s, w])
    else:
        i = int(np.argmax(np.diag(R)))
        j, k = (i + 1) % 3, (i + 2) % 3
        s = np.sqrt(R[i, i] - R[j, j] - R[k, k] + 1.0)
        v = np.zeros(3)
        v[i] = 0.5 * s
        s = 0.5 / s
        w = (R[k, j] - R[j, k]) * s
        v[j] = (R[j, i] + R[i, j]) * s
        v[k] = (R[k, i] + R[i, k]) * s
        q = np.array([v[0], v[1], v[2], w])
    if q[3] < 0:
        q = -q
    return q / np.linalg.norm(q)


def _qbatch(R):
    """Vectorised form of _q1 (all four branches evaluated, one selected per row)."""
    tr = np.trace(R, axis1=1, axis2=2)
    d = np.stack([R[:, 0, 0], R[:, 1, 1], R[:, 2, 2]], 1)
    out = np.zeros((len(R), 4))
    use_tr = tr > 0
    s = np.sqrt(np.maximum(tr, 0) + 1.0)
    inv = 0.5 / s
    qt = np.stack([(R[:, 2, 1] - R[:, 1, 2]) * inv, (R[:, 0, 2] - R[:, 2, 0]) * inv,
                   (R[:, 1, 0] - R[:, 0, 1]) * inv, 0.5 * s], 1)
    out[use_tr] = qt[use_tr]
    for i in range(3):
        j, k = (i + 1) % 3, (i + 2) % 3
        sel = (~use_tr) & (np.argmax(d, 1) == i)
        if not sel.any():
            continue
        Rs = R[sel]
        si = np.sqrt(Rs[:, i, i] - Rs[:, j, j] - Rs[:, k, k] + 1.0)
        inv = 0.5 / si
        q = np.zeros((len(Rs), 4))
        q[:, i] = 0.5 * si
        q[:, 3] = (Rs[:, k, j] - Rs[:, j, k]) * inv
        q[:, j] = (Rs[:, j, i] + Rs[:, i, j]) * inv
        q[:, k] = (Rs[:, k, i] + Rs[:, i, k]) * inv
        out[sel] = q
    out[out[:, 3] < 0] *= -1
    return out / np.linalg.norm(out, axis=1, keepdims=True)


@pytest.fixture(scope="module")
def edges():
    T_bw, T_cb, K, X, obs, cam = synth.random_edges(N_EDGES, seed=3000)
    qb = np.concatenate([_qbatch(T_bw[:, :3, :3]), T_bw[:, :3, 3]], 1)
    qc3 = np.stack([np.concatenate([_q1(T[:3, :3]), T[:3, 3]]) for T in synth.baseline_rig().T_cb])
    qc = qc3[cam]
    return dict(T_bw=T_bw, T_cb=T_cb, K=K, X=X, obs=obs, cam=cam, qb=qb, qc=qc)


def _torch(e, dtype):
    import torch
    f = lambda a: torch.as_tensor(a, dtype=dtype, device="cuda").contiguous()
    return f(e["qb"]), f(e["qc"]), f(e["X"]), f(e["K"]), f(e["obs"])


def test_forward_matches_fp64_numpy(edges, gpu):
    torch = pytest.importorskip("torch")
    from mcvslam_gb300.autograd import reprojection_residual
    qb, qc, X, K, obs = _torch(edges, torch.float64)
    r = reprojection_residual(qb, qc, X, K, obs).cpu().numpy()
    Tcw = edges["T_cb"] @ edges["T_bw"]
    Pc = np.einsum("nij,nj->ni", Tcw[:, :3, :3], edges["X"]) + Tcw[:, :3, 3]
    uv = np.stack([edges["K"][:, 0] * Pc[:, 0] / Pc[:, 2] + edges["K"][:, 2],
                   edges["K"][:, 1] * Pc[:, 1] / Pc[:, 2] + edges["K"][:, 3]], 1)
    np.testing.assert_allclose(r, edges["obs"] - uv, rtol=0, atol=1e-8)
    qb32, qc32, X32, K32, obs32 = _torch(edges, torch.float32)
    r32 = reprojection_residual(qb32, qc32, X32, K32, obs32).cpu().numpy()
    assert np.abs(r32 - r).max() < 0.05  # pixels; FP32 of world coordinates ~10 m


@pytest.mark.parametrize("dtype_name", ["float64", "float32"])
def test_backward_matches_central_differences(edges, dtype_name, gpu):
    torch = pytest.importorskip("torch")
    from mcvslam_gb300.autograd import reprojection_residual
    dtype = getattr(torch, dtype_name)
    qb, qc, X, K, obs = _torch(edges, dtype)
    n = X.shape[0]
    g = torch.randn((n, 2), dtype=dtype, device="cuda")
    dp = torch.zeros((n, 6), dtype=dtype, device="cuda", requires_grad=True)
    de = torch.zeros((n, 6), dtype=dtype, device="cuda", requires_grad=True)
    Xr = X.clone().requires_grad_(True)
    r = reprojection_residual(qb, qc, Xr, K, obs, dp, de)
    (r * g).sum().backward()
    # FD reference always in FP64 on a subset of edges
    sub = slice(0, 20000)
    qb64, qc64, X64, K64, obs64 = [t[sub] for t in _torch(edges, torch.float64)]
    g64 = g[sub].double()
    h = 1e-6
    m = X64.shape[0]

    def f(dp_, de_, X_):
        return (reprojection_residual(qb64, qc64, X_, K64, obs64, dp_, de_) * g64).sum(1)

    zeros6 = torch.zeros((m, 6), dtype=torch.float64, device="cuda")
    fd_p = torch.zeros((m, 6), dtype=torch.float64, device="cuda")
    fd_e = torch.zeros((m, 6), dtype=torch.float64, device="cuda")
    fd_x = torch.zeros((m, 3), dtype=torch.float64, device="cuda")
    for k in range(6):
        d = zeros6.clone()
        d[:, k] = h
        fd_p[:, k] = (f(d, zeros6, X64) - f(-d, zeros6, X64)) / (2 * h)
        fd_e[:, k] = (f(zeros6, d, X64) - f(zeros6, -d, X64)) / (2 * h)
    for k in range(3):
        d = torch.zeros_like(X64)
        d[:, k] = h
        fd_x[:, k] = (f(zeros6, zeros6, X64 + d) - f(zeros6, zeros6, X64 - d)) / (2 * h)
    tol = 2e-5 if dtype_name == "float64" else 2e-3
    for got, ref in ((dp.grad[sub].double(), fd_p), (de.grad[sub].double(), fd_e), (Xr.grad[sub].double(), fd_x)):
        scale = ref.abs().max(1, keepdim=True).values + 1e-12
        err = ((got - ref).abs() / scale).max().item()
        assert err < tol, err


def test_jacobians_match_oracle_linearize(edges, gpu):
    torch = pytest.importorskip("torch")
    from mcvslam_gb300.autograd import jacobians
    m = 20000
    rig = synth.baseline_rig()
    # the same edges as an oracle problem: one pose and one point per edge
    T_bw32 = edges["T_bw"][:m].astype(np.float32)
    pr = synth.Problem(
        cam_K=rig.K, cam_bf=rig.bf, cam_Tcb=rig.T_cb.astype(np.float32).reshape(-1, 16), cam_size=rig.size,
        pose_Tcw=T_bw32.reshape(m, 16), pose_fixed=np.zeros(m, np.uint8),
        point_Xw=edges["X"][:m].astype(np.float32), point_fixed=np.zeros(m, np.uint8),
        edge_type=np.zeros(m, np.uint8), edge_pose=np.arange(m, dtype=np.int32),
        edge_point=np.arange(m, dtype=np.int32), edge_cam=edges["cam"][:m].astype(np.int32),
        edge_obs=np.concatenate([edges["obs"][:m], np.zeros((m, 1))], 1).astype(np.float32),
        edge_info=np.ones(m, np.float32), edge_delta=np.full(m, 2.0, np.float32),
        edge_robust=np.ones(m, np.uint8), edge_level=np.zeros(m, np.uint8))
    err, Jl, Jp = oracle.linearize_edges(pr)
    # identical FP64 state on the device: the oracle's conversions of the float inputs
    qb = np.stack([oracle.mat44f_to_qt(T) for T in T_bw32])
    qc3 = np.stack([oracle.mat44f_to_qt(T) for T in rig.T_cb.astype(np.float32)])
    f = lambda a: torch.as_tensor(a, dtype=torch.float64, device="cuda").contiguous()
    Kd = f(rig.K.astype(np.float64)[edges["cam"][:m]])
    Jpose, Jext, JX = jacobians(f(qb), f(qc3[edges["cam"][:m]]), f(pr.point_Xw.astype(np.float64)), Kd)
    np.testing.assert_allclose(Jpose.cpu().numpy(), Jp[:, :2], rtol=1e-9, atol=1e-9 * np.abs(Jp).max())
    np.testing.assert_allclose(JX.cpu().numpy(), Jl[:, :2], rtol=1e-9, atol=1e-9 * np.abs(Jl).max())


def test_reproj_rejects_wrong_shapes(gpu):
    torch = pytest.importorskip("torch")
    from mcvslam_gb300.autograd import reprojection_residual
    z = torch.zeros((4, 7), dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError):
        reprojection_residual(z, z, torch.zeros((4, 2), dtype=torch.float64, device="cuda"),
                              torch.zeros((4, 4), dtype=torch.float64, device="cuda"),
                              torch.zeros((4, 2), dtype=torch.float64, device="cuda"))
