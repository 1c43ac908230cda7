"""Known-answer tests of the CPU oracle (hand-derived values, closed forms)."""
import math

import numpy as np
import pytest

from mcvslam_gb300 import synth
from oracle import oracle


def skew(w):
    return np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])


def R_of_qt(qt):
    return oracle.qt_to_mat44f(qt).astype(np.float64)[:3, :3]


def rodrigues(w):
    th = np.linalg.norm(w)
    if th == 0:
        return np.eye(3)
    K = skew(w / th)
    return np.eye(3) + math.sin(th) * K + (1 - math.cos(th)) * K @ K


def quat_to_R(q):
    x, y, z, w = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


@pytest.mark.parametrize("theta", [0.0, 1e-6, 0.5, math.pi - 1e-6])
def test_se3_exp_closed_form(theta):
    axis = np.array([0.3, -0.5, 0.8])
    axis /= np.linalg.norm(axis)
    w = axis * theta
    v = np.array([0.2, -1.0, 0.7])
    qt = oracle.se3_exp(np.concatenate([w, v]))
    assert qt[3] >= 0 and abs(np.linalg.norm(qt[:4]) - 1) < 1e-15
    R = quat_to_R(qt[:4])
    np.testing.assert_allclose(R, rodrigues(w), atol=1e-12)
    # V = I + (1-cos)/th^2 W + (th - sin)/th^3 W^2 (series below 1e-5)
    W = skew(w)
    if theta < 1e-5:
        V = np.eye(3) + 0.5 * W + W @ W / 6
    else:
        V = np.eye(3) + (1 - math.cos(theta)) / theta**2 * W + (theta - math.sin(theta)) / theta**3 * W @ W
    np.testing.assert_allclose(qt[4:], V @ v, atol=1e-12)


def test_quaternion_of_matrix_all_branches():
    rng = np.random.default_rng(0)
    Rs = list(synth.random_rotations(rng, 200)) + [np.diag([1.0, -1, -1]), np.diag([-1.0, 1, -1]),
                                                   np.diag([-1.0, -1, 1]), np.eye(3)]
    for R in Rs:
        T = np.eye(4, dtype=np.float32)
        T[:3, :3] = R
        T[:3, 3] = [1, 2, 3]
        qt = oracle.mat44f_to_qt(T)
        assert qt[3] >= 0
        np.testing.assert_allclose(quat_to_R(qt[:4]), T[:3, :3].astype(np.float64), atol=2e-7)
        np.testing.assert_array_equal(qt[4:], [1, 2, 3])


def test_huber_kernel():
    d = float(np.float32(math.sqrt(5.991)))
    for e2 in [0.0, 1.0, d * d * (1 - 1e-12), d * d, d * d * (1 + 1e-12), 100.0]:
        rho = oracle.huber(e2, d)
        if e2 <= d * d:
            np.testing.assert_array_equal(rho, [e2, 1.0, 0.0])
        else:
            s = math.sqrt(e2)
            np.testing.assert_allclose(rho, [2 * s * d - d * d, d / s, -0.5 * (d / s) / e2], rtol=1e-15)
    # continuity of rho and rho' at the threshold
    a, b = oracle.huber(d * d, d), oracle.huber(d * d * (1 + 1e-9), d)
    assert abs(a[0] - b[0]) < 1e-6 and abs(a[1] - b[1]) < 1e-6


def test_compose_and_map():
    rng = np.random.default_rng(1)
    R1, R2 = synth.random_rotations(rng, 2)
    t1, t2 = rng.normal(size=3), rng.normal(size=3)

    def qt(R, t):
        T = np.eye(4, dtype=np.float32)
        T[:3, :3] = R
        T[:3, 3] = t
        return oracle.mat44f_to_qt(T)

    a, b = qt(R1, t1), qt(R2, t2)
    c = oracle.compose(a, b)
    Ra, Rb = quat_to_R(a[:4]), quat_to_R(b[:4])
    np.testing.assert_allclose(quat_to_R(c[:4]), Ra @ Rb, atol=1e-14)
    np.testing.assert_allclose(c[4:], Ra @ b[4:] + a[4:], atol=1e-14)
    X = np.array([0.5, -2.0, 7.0])
    np.testing.assert_allclose(oracle.map_point(a, X), Ra @ X + a[4:], atol=1e-13)


def _residual_mono(qt_pose, qt_cb, X, K):
    Pb = quat_to_R(qt_pose[:4]) @ X + qt_pose[4:]
    Pc = quat_to_R(qt_cb[:4]) @ Pb + qt_cb[4:]
    return np.array([K[0] * Pc[0] / Pc[2] + K[2], K[1] * Pc[1] / Pc[2] + K[3]])


def _residual_stereo(qt_pose, X, K, bf):
    Pc = quat_to_R(qt_pose[:4]) @ X + qt_pose[4:]
    u = K[0] * Pc[0] / Pc[2] + K[2]
    return np.array([u, K[1] * Pc[1] / Pc[2] + K[3], u - bf / Pc[2]])


def _left(qt, d):
    return oracle.compose(oracle.se3_exp(d), qt)


def test_jacobians_against_central_differences():
    pr = synth.reference_style(seed=3, n_kf=3, n_points=60)
    err, Jl, Jp = oracle.linearize_edges(pr)
    h = 1e-6
    checked = {0: 0, 1: 0}
    for i in range(pr.n_edges):
        t = int(pr.edge_type[i])
        if checked.get(t, 99) >= 20:
            continue
        checked[t] += 1
        qt = oracle.mat44f_to_qt(pr.pose_Tcw[pr.edge_pose[i]])
        X = pr.point_Xw[pr.edge_point[i]].astype(np.float64)
        K = pr.cam_K[pr.edge_cam[i]].astype(np.float64)
        cb = oracle.mat44f_to_qt(pr.cam_Tcb[pr.edge_cam[i]])
        if t == 0:
            f = lambda q, x: pr.edge_obs[i, :2].astype(np.float64) - _residual_mono(q, cb, x, K)
            dim = 2
        else:
            f = lambda q, x: pr.edge_obs[i].astype(np.float64) - _residual_stereo(q, x, K, float(pr.cam_bf[pr.edge_cam[i]]))
            dim = 3
        Jp_fd = np.zeros((dim, 6))
        for k in range(6):
            d = np.zeros(6)
            d[k] = h
            Jp_fd[:, k] = (f(_left(qt, d), X) - f(_left(qt, -d), X)) / (2 * h)
        Jl_fd = np.zeros((dim, 3))
        for k in range(3):
            d = np.zeros(3)
            d[k] = h
            Jl_fd[:, k] = (f(qt, X + d) - f(qt, X - d)) / (2 * h)
        scale = np.abs(Jp_fd).max()
        np.testing.assert_allclose(Jp[i, :dim], Jp_fd, atol=2e-5 * scale)
        np.testing.assert_allclose(Jl[i, :dim], Jl_fd, atol=2e-5 * np.abs(Jl_fd).max())
    assert checked[0] > 0 and checked[1] > 0


def test_stereo_invz_is_float_rounded():
    pr = synth.reference_style(seed=4, n_kf=2, n_points=40)
    err, _, _ = oracle.linearize_edges(pr)
    idx = np.nonzero(pr.edge_type == 1)[0]
    assert len(idx)
    for i in idx[:10]:
        qt = oracle.mat44f_to_qt(pr.pose_Tcw[pr.edge_pose[i]])
        K = pr.cam_K[0].astype(np.float64)
        Pc = quat_to_R(qt[:4]) @ pr.point_Xw[pr.edge_point[i]].astype(np.float64) + qt[4:]
        invz = float(np.float32(1.0 / Pc[2]))
        u = Pc[0] * invz * K[0] + K[2]
        v = Pc[1] * invz * K[1] + K[3]
        ur = u - float(np.float32(np.float32(pr.cam_bf[0]) * np.float32(invz)))
        np.testing.assert_allclose(err[i], pr.edge_obs[i].astype(np.float64) - [u, v, ur], rtol=0, atol=1e-9)


def test_schur_solution_equals_full_solve():
    pr = synth.local_ba(5, 150, seed=11)
    for lam in [1e-3, 1.0, 1e3]:
        H, b, x = oracle.normal_equations(pr, lam)
        np.testing.assert_allclose(x, np.linalg.solve(H, b), rtol=1e-8, atol=1e-12 * np.abs(x).max())


def test_lambda_init_and_gain_ratio_on_toy():
    """First LM trial of a 3-pose toy: lambda0 = 1e-5 * max diag(H), rho from the
    model decrease x^T(lambda x + b), all recomputed here from the normal equations."""
    pr = synth.local_ba(3, 40, seed=5, n_fixed=1)
    r = oracle.optimize(pr, 1)
    H, b, x = oracle.normal_equations(pr, 0.0)
    lam0 = 1e-5 * np.abs(np.diag(H)).max()
    first = r["log"][0]
    assert first["lambda"] == pytest.approx(lam0, rel=1e-12)
    H2, b2, x2 = oracle.normal_equations(pr, lam0)
    scale = x2 @ (lam0 * x2 + b2) + 1e-3
    assert first["scale"] == pytest.approx(scale, rel=1e-9)
    assert first["rho"] == pytest.approx((first["chi_before"] - first["chi_after"]) / scale, rel=1e-12)


def test_pose_optimization_rounds_logic():
    pr = synth.pose_only(300, seed=9)
    r = oracle.pose_optimization(pr, rounds=4, iters=10, chi2_thr=5.991)
    lv = r["edge_level"]
    # outliers are never re-admitted; inlier count = edges - newly rejected in the last round
    assert lv.sum() > 0.05 * pr.n_edges
    assert r["ret"] <= pr.n_edges and r["pose_written"] == 1
    gt = pr.gt_pose_Tcw[0]
    T = oracle.qt_to_mat44f(r["pose_qt"][0]).astype(np.float64)
    assert np.linalg.norm(T[:3, 3] - gt[:3, 3]) < 0.02


def test_pose_optimization_too_few_edges():
    pr = synth.pose_only(2, seed=9)
    r = oracle.pose_optimization(pr)
    assert r["ret"] == 0


def test_local_ba_filter_and_return_value():
    pr = synth.config(1)
    r = oracle.local_ba(pr, 10)
    assert r["ret"] == pr.n_edges and r["written"] == 1
    # every edge that ends above the threshold was set to level 1
    assert np.all(r["edge_level"][r["edge_chi2"].astype(np.float32) >= np.float32(5.991)] == 1)


def test_threaded_oracle_matches_serial():
    pr = synth.local_ba(8, 600, seed=21)
    a = oracle.optimize(pr, 5, n_threads=1)
    b = oracle.optimize(pr, 5, n_threads=4)
    np.testing.assert_allclose(a["pose_qt"], b["pose_qt"], rtol=0, atol=1e-9)
    assert abs(a["final_chi2"] - b["final_chi2"]) <= 1e-9 * a["final_chi2"]
