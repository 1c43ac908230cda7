"""Generates tests/golden/ba_kat.json: known answers computed at 50 significant
digits with mpmath, independently of the oracle and of the CUDA kernels.

The reference (MCVSLAM + its vendored g2o) publishes no golden vectors for
the bundle-adjustment path and cannot be built here, so these fixtures pin
the arithmetic both implementations must share to the published formulas
the reference's code follows:

  * SE3Quat::exp (ThirdParty/g2o/g2o/types/slam3d/se3quat.h:218-257): the
    second-order series below theta = 1e-5, Rodrigues above, then
    Quaternion(R) (Shoemake's trace / largest-diagonal method) and the
    w >= 0 normalisation;
  * the float 4x4 -> SE3Quat conversion (src/Converter.cc:31-45);
  * the mono reprojection residual and its Jacobians
    (include/OptimizeTypes.hpp:80-113, modules/camera/Pinhole.cpp:55-60,105-116);
  * the Huber kernel (ThirdParty/g2o/g2o/core/robust_kernel_impl.cpp:65-78);
  * the first Levenberg-Marquardt trial of a small problem: robustified
    normal equations (base_binary_edge.hpp:64-136 with W = rho' Omega,
    base_edge.h:143-149), lambda_0 = tau max|H_jj| over poses and points
    (optimization_algorithm_levenberg.cpp:145-157), the damped solve, the
    SE3 exp / additive update, the new robust chi2 and the gain ratio
    (:93-131, :159-165).  The full system is solved directly; the Schur
    complement gives the same solution.

Run with the repository root on sys.path:  python tests/golden/make_golden.py
(needs mpmath, which is not needed to run the tests).
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np
import mpmath as mp

mp.mp.dps = 50
HERE = os.path.dirname(os.path.abspath(__file__))


def M(a):
    return mp.matrix([[mp.mpf(float(v)) for v in row] for row in a])


def skew(w):
    return mp.matrix([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])


def quat_of_R(m):
    """Shoemake's method as in Eigen's Quaternion(Matrix3), then g2o's
    normalizeRotation (w >= 0, unit norm).  Returns (x, y, z, w)."""
    t = m[0, 0] + m[1, 1] + m[2, 2]
    q = [mp.mpf(0)] * 4  # x y z w
    if t > 0:
        t = mp.sqrt(t + 1)
        q[3] = t / 2
        t = mp.mpf(1) / (2 * t)
        q[0] = (m[2, 1] - m[1, 2]) * t
        q[1] = (m[0, 2] - m[2, 0]) * t
        q[2] = (m[1, 0] - m[0, 1]) * t
    else:
        i = 0
        if m[1, 1] > m[0, 0]:
            i = 1
        if m[2, 2] > m[i, i]:
            i = 2
        j = (i + 1) % 3
        k = (j + 1) % 3
        t = mp.sqrt(m[i, i] - m[j, j] - m[k, k] + 1)
        q[i] = t / 2
        t = mp.mpf(1) / (2 * t)
        q[3] = (m[k, j] - m[j, k]) * t
        q[j] = (m[j, i] + m[i, j]) * t
        q[k] = (m[k, i] + m[i, k]) * t
    if q[3] < 0:
        q = [-v for v in q]
    n = mp.sqrt(sum(v * v for v in q))
    return [v / n for v in q]


def R_of_quat(q):
    x, y, z, w = q
    return mp.matrix([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                      [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                      [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def se3_exp(u):
    w = mp.matrix([u[0], u[1], u[2]])
    ups = mp.matrix([u[3], u[4], u[5]])
    th = mp.sqrt(w[0] ** 2 + w[1] ** 2 + w[2] ** 2)
    O = skew(w)
    O2 = O * O
    I = mp.eye(3)
    if th < mp.mpf("0.00001"):
        R = I + O + O2 / 2
        V = I + O / 2 + O2 / 6
    else:
        R = I + mp.sin(th) / th * O + (1 - mp.cos(th)) / th ** 2 * O2
        V = I + (1 - mp.cos(th)) / th ** 2 * O + (th - mp.sin(th)) / th ** 3 * O2
    return quat_of_R(R), V * ups


def compose(qa, ta, qb, tb):
    """(a * b): q = qa qb (normalised, w >= 0), t = Ra tb + ta."""
    x1, y1, z1, w1 = qa
    x2, y2, z2, w2 = qb
    q = [w1 * x2 + x1 * w2 + y1 * z2 - z1 * y2,
         w1 * y2 - x1 * z2 + y1 * w2 + z1 * x2,
         w1 * z2 + x1 * y2 - y1 * x2 + z1 * w2,
         w1 * w2 - x1 * x2 - y1 * y2 - z1 * z2]
    if q[3] < 0:
        q = [-v for v in q]
    n = mp.sqrt(sum(v * v for v in q))
    q = [v / n for v in q]
    return q, R_of_quat(qa) * tb + ta


def se3_of_mat44f(T):
    T = np.asarray(T, np.float32).reshape(4, 4)
    R = M(T[:3, :3])
    t = mp.matrix([mp.mpf(float(v)) for v in T[:3, 3]])
    return quat_of_R(R), t


def huber(e2, delta):
    d2 = delta * delta
    if e2 <= d2:
        return e2, mp.mpf(1)
    s = mp.sqrt(e2)
    return 2 * s * delta - d2, delta / s


def mono_edge(q_bw, t_bw, q_cb, t_cb, K, X, obs):
    """Residual e = z - pi(T_cb T_bw X) and Jacobians w.r.t. the body pose
    (left perturbation, rotation first) and the point."""
    fx, fy, cx, cy = K
    R_bw = R_of_quat(q_bw)
    R_cb = R_of_quat(q_cb)
    Pb = R_bw * X + t_bw
    Pc = R_cb * Pb + t_cb
    x, y, z = Pc[0], Pc[1], Pc[2]
    u = fx * x / z + cx
    v = fy * y / z + cy
    e = mp.matrix([obs[0] - u, obs[1] - v])
    Jpi = mp.matrix([[fx / z, 0, -fx * x / z ** 2], [0, fy / z, -fy * y / z ** 2]])
    Jl = -Jpi * R_cb * R_bw
    A = mp.matrix(3, 6)
    S = -skew(Pb)
    for r in range(3):
        for c in range(3):
            A[r, c] = S[r, c]
        A[r, 3 + r] = 1
    Jp = -Jpi * R_cb * A
    return e, Jp, Jl


def tiny_problem():
    """One fixed and one free keyframe, 5 free points, 2 cameras, 10 mono
    edges, one gross outlier (Huber's linear branch)."""
    rng = np.random.default_rng(20240611)
    cams_K = np.array([[500.0, 500.0, 320.0, 240.0], [450.0, 455.0, 330.0, 250.0]], np.float32)
    Tcb = np.tile(np.eye(4, dtype=np.float32), (2, 1, 1))
    c, s = np.cos(0.3), np.sin(0.3)
    Tcb[1, :3, :3] = np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]], np.float32)
    Tcb[1, :3, 3] = [-0.4, 0.0, 0.05]
    poses = np.tile(np.eye(4, dtype=np.float32), (2, 1, 1))
    a = 0.05
    poses[1, :3, :3] = np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1]], np.float32)
    poses[1, :3, 3] = [-0.3, 0.02, 0.01]
    X_true = np.array([[0.2, 0.1, 4.0], [-0.5, 0.3, 5.0], [0.7, -0.2, 6.0], [0.1, 0.5, 3.5], [-0.2, -0.4, 4.5]])
    edges = []
    for k in range(2):
        for cam in range(2):
            for p in range(5):
                if (k + cam + p) % 2:
                    continue
                edges.append((k, p, cam))
    obs = []
    for (k, p, cam) in edges:
        T = poses[k].astype(np.float64)
        Pc = Tcb[cam].astype(np.float64) @ (T @ np.append(X_true[p], 1.0))
        fx, fy, cx, cy = cams_K[cam].astype(np.float64)
        obs.append([fx * Pc[0] / Pc[2] + cx + rng.normal(0, 1), fy * Pc[1] / Pc[2] + cy + rng.normal(0, 1), 0.0])
    obs = np.array(obs, np.float32)
    obs[3, :2] += np.array([25.0, -18.0], np.float32)  # outlier
    X_init = (X_true + rng.normal(0, 0.05, X_true.shape)).astype(np.float32)
    poses_init = poses.copy()
    poses_init[1, :3, 3] += np.array([0.02, -0.01, 0.015], np.float32)
    return {
        "cam_K": cams_K.tolist(), "cam_Tcb": Tcb.reshape(2, 16).tolist(),
        "pose_Tcw": poses_init.reshape(2, 16).tolist(), "pose_fixed": [1, 0],
        "point_Xw": X_init.tolist(),
        "edge_pose": [e[0] for e in edges], "edge_point": [e[1] for e in edges], "edge_cam": [e[2] for e in edges],
        "edge_obs": obs.tolist(), "edge_info": [1.0] * len(edges),
        "edge_delta": [float(np.float32(np.sqrt(5.991)))] * len(edges),
    }


def first_trial(P):
    """robust chi2, lambda_0, damped solve, new chi2, gain ratio of the first
    LM trial; free pose 1 first, then the 5 points (g2o's index order)."""
    K = [[mp.mpf(v) for v in k] for k in P["cam_K"]]
    cams = [se3_of_mat44f(np.array(t, np.float32)) for t in P["cam_Tcb"]]
    poses = [se3_of_mat44f(np.array(t, np.float32)) for t in P["pose_Tcw"]]
    pts = [mp.matrix([mp.mpf(v) for v in x]) for x in P["point_Xw"]]
    nE = len(P["edge_pose"])
    delta = mp.mpf(P["edge_delta"][0])

    def chi2_of(poses_, pts_):
        tot = mp.mpf(0)
        for i in range(nE):
            k, p, c = P["edge_pose"][i], P["edge_point"][i], P["edge_cam"][i]
            obs = [mp.mpf(v) for v in P["edge_obs"][i][:2]]
            e, _, _ = mono_edge(poses_[k][0], poses_[k][1], cams[c][0], cams[c][1], K[c], pts_[p], obs)
            e2 = (e[0] ** 2 + e[1] ** 2) * mp.mpf(P["edge_info"][i])
            tot += huber(e2, delta)[0]
        return tot

    n = 6 + 3 * 5
    H = mp.zeros(n, n)
    b = mp.zeros(n, 1)
    for i in range(nE):
        k, p, c = P["edge_pose"][i], P["edge_point"][i], P["edge_cam"][i]
        obs = [mp.mpf(v) for v in P["edge_obs"][i][:2]]
        e, Jp, Jl = mono_edge(poses[k][0], poses[k][1], cams[c][0], cams[c][1], K[c], pts[p], obs)
        info = mp.mpf(P["edge_info"][i])
        e2 = (e[0] ** 2 + e[1] ** 2) * info
        w = huber(e2, delta)[1] * info
        J = mp.zeros(2, n)
        if k == 1:
            for r in range(2):
                for q in range(6):
                    J[r, q] = Jp[r, q]
        for r in range(2):
            for q in range(3):
                J[r, 6 + 3 * p + q] = Jl[r, q]
        H += J.T * J * w
        b += -(J.T * e) * w
    lam = mp.mpf("1e-5") * max(abs(H[j, j]) for j in range(n))
    Hd = H + lam * mp.eye(n)
    x = mp.lu_solve(Hd, b)
    chi0 = chi2_of(poses, pts)
    q1, t1 = se3_exp([x[j] for j in range(6)])
    new_poses = [poses[0], compose(q1, t1, poses[1][0], poses[1][1])]
    new_pts = [pts[p] + mp.matrix([x[6 + 3 * p + q] for q in range(3)]) for p in range(5)]
    chi1 = chi2_of(new_poses, new_pts)
    scale = sum(x[j] * (lam * x[j] + b[j]) for j in range(n)) + mp.mpf("1e-3")
    rho = (chi0 - chi1) / scale
    return {"chi_before": chi0, "chi_after": chi1, "lambda": lam, "scale": scale, "rho": rho,
            "x": [x[j] for j in range(n)], "H_diag": [H[j, j] for j in range(n)], "b": [b[j] for j in range(n)]}


def s(v):
    return mp.nstr(v, 30)


def main():
    out = {"generator": "tests/golden/make_golden.py (mpmath, 50 digits)", "se3_exp": [], "huber": [],
           "mono_edges": [], "lm_first_trial": {}}
    axis = np.array([0.3, -0.5, 0.8]) / np.linalg.norm([0.3, -0.5, 0.8])
    for th in [0.0, 1e-6, 9.9e-6, 1e-3, 0.5, 2.0, np.pi - 1e-6]:
        u = [float(v) for v in axis * th] + [0.2, -1.0, 0.7]
        q, t = se3_exp([mp.mpf(v) for v in u])
        out["se3_exp"].append({"u": u, "q_xyzw": [s(v) for v in q], "t": [s(t[i]) for i in range(3)]})
    for e2, d in [(0.5, 2.0), (4.0, 2.0), (4.0000001, 2.0), (50.0, 2.44744754), (1e6, 2.79553223)]:
        r0, r1 = huber(mp.mpf(e2), mp.mpf(d))
        out["huber"].append({"e2": e2, "delta": d, "rho0": s(r0), "rho1": s(r1)})
    P = tiny_problem()
    out["problem"] = P
    K = [[mp.mpf(v) for v in k] for k in P["cam_K"]]
    cams = [se3_of_mat44f(np.array(t, np.float32)) for t in P["cam_Tcb"]]
    poses = [se3_of_mat44f(np.array(t, np.float32)) for t in P["pose_Tcw"]]
    for i in range(len(P["edge_pose"])):
        k, p, c = P["edge_pose"][i], P["edge_point"][i], P["edge_cam"][i]
        X = mp.matrix([mp.mpf(v) for v in P["point_Xw"][p]])
        e, Jp, Jl = mono_edge(poses[k][0], poses[k][1], cams[c][0], cams[c][1], K[c], X,
                              [mp.mpf(v) for v in P["edge_obs"][i][:2]])
        out["mono_edges"].append({"e": [s(e[r]) for r in range(2)],
                                  "J_pose": [[s(Jp[r, q]) for q in range(6)] for r in range(2)],
                                  "J_point": [[s(Jl[r, q]) for q in range(3)] for r in range(2)]})
    out["pose_qt"] = [[s(v) for v in q] + [s(t[i]) for i in range(3)] for q, t in poses]
    ft = first_trial(P)
    out["lm_first_trial"] = {k: ([s(v) for v in val] if isinstance(val, list) else s(val)) for k, val in ft.items()}
    with open(os.path.join(HERE, "ba_kat.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", os.path.join(HERE, "ba_kat.json"))


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    main()
