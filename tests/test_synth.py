import numpy as np

from mcvslam_gb300 import synth


def test_generator_is_deterministic():
    a, b = synth.config(1), synth.config(1)
    for k, v in a.arrays().items():
        np.testing.assert_array_equal(v, getattr(b, k))


def test_config_sizes():
    p1 = synth.config(1)
    assert 8000 <= p1.n_edges <= 11000
    cnt = np.bincount(p1.edge_point)
    assert cnt.min() >= 2 and cnt.max() <= 8
    p2 = synth.config(2)
    assert 130000 <= p2.n_edges <= 170000 and p2.n_poses == 30
    assert p2.pose_fixed[:2].all() and not p2.pose_fixed[2:].any()


def test_outlier_fraction_and_noise():
    p = synth.config(2)
    proj_err = []
    # reprojection error at the ground truth: ~N(0,1) for inliers, large for ~5% outliers
    T = p.gt_pose_Tcw
    for c in range(3):
        idx = np.nonzero(p.edge_cam == c)[0][:3000]
        Tcb = p.cam_Tcb[c].reshape(4, 4).astype(np.float64)
        Tcw = Tcb @ T[p.edge_pose[idx]]
        Pc = np.einsum("nij,nj->ni", Tcw[:, :3, :3], p.gt_point_Xw[p.edge_point[idx]]) + Tcw[:, :3, 3]
        K = p.cam_K[c].astype(np.float64)
        uv = np.stack([K[0] * Pc[:, 0] / Pc[:, 2] + K[2], K[1] * Pc[:, 1] / Pc[:, 2] + K[3]], 1)
        proj_err.append(np.linalg.norm(uv - p.edge_obs[idx, :2], axis=1))
    e = np.concatenate(proj_err)
    out = (e > 6).mean()
    assert 0.03 < out < 0.08
    assert 1.0 < np.median(e) < 1.5
