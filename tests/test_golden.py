"""Oracle (CPU) and CUDA path against the 50-digit fixtures of
tests/golden/ba_kat.json (generated by tests/golden/make_golden.py)."""
import json
import os

import numpy as np
import pytest

from mcvslam_gb300 import synth
from oracle import oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ba_kat.json")


@pytest.fixture(scope="module")
def kat():
    with open(GOLDEN) as f:
        return json.load(f)


def problem(P) -> synth.Problem:
    E = len(P["edge_pose"])
    return synth.Problem(
        cam_K=np.array(P["cam_K"], np.float32), cam_bf=np.zeros(2, np.float32),
        cam_Tcb=np.array(P["cam_Tcb"], np.float32), cam_size=np.array([[640, 480]] * 2, np.int32),
        pose_Tcw=np.array(P["pose_Tcw"], np.float32), pose_fixed=np.array(P["pose_fixed"], np.uint8),
        point_Xw=np.array(P["point_Xw"], np.float32), point_fixed=np.zeros(len(P["point_Xw"]), np.uint8),
        edge_type=np.zeros(E, np.uint8), edge_pose=np.array(P["edge_pose"], np.int32),
        edge_point=np.array(P["edge_point"], np.int32), edge_cam=np.array(P["edge_cam"], np.int32),
        edge_obs=np.array(P["edge_obs"], np.float32), edge_info=np.array(P["edge_info"], np.float32),
        edge_delta=np.array(P["edge_delta"], np.float32), edge_robust=np.ones(E, np.uint8),
        edge_level=np.zeros(E, np.uint8), name="golden_tiny")


def test_se3_exp_matches_50_digit_values(kat):
    for case in kat["se3_exp"]:
        qt = oracle.se3_exp(np.array(case["u"]))
        np.testing.assert_allclose(qt[:4], [float(v) for v in case["q_xyzw"]], rtol=0, atol=2e-16)
        # (theta - sin theta) / theta^3 cancels in double below theta ~ 1e-2,
        # exactly as in the reference's formula: a few 1e-15 absolute on t
        np.testing.assert_allclose(qt[4:7], [float(v) for v in case["t"]], rtol=0, atol=2e-14)


def test_huber_matches_50_digit_values(kat):
    for case in kat["huber"]:
        rho = oracle.huber(case["e2"], case["delta"])
        assert rho[0] == pytest.approx(float(case["rho0"]), rel=1e-15)
        assert rho[1] == pytest.approx(float(case["rho1"]), rel=1e-15)


def test_float_pose_conversion_matches_50_digit_values(kat):
    P = kat["problem"]
    for T, ref in zip(P["pose_Tcw"], kat["pose_qt"]):
        qt = oracle.mat44f_to_qt(np.array(T, np.float32))
        np.testing.assert_allclose(qt[:7], [float(v) for v in ref], rtol=0, atol=2e-16)


def test_mono_residual_and_jacobians_match_50_digit_values(kat):
    pr = problem(kat["problem"])
    err, Jl, Jp = oracle.linearize_edges(pr)
    for i, ref in enumerate(kat["mono_edges"]):
        np.testing.assert_allclose(err[i, :2], [float(v) for v in ref["e"]], rtol=1e-12, atol=1e-11)
        np.testing.assert_allclose(Jp[i, :2], np.array(ref["J_pose"], dtype=np.float64), rtol=1e-12, atol=1e-10)
        np.testing.assert_allclose(Jl[i, :2], np.array(ref["J_point"], dtype=np.float64), rtol=1e-12, atol=1e-10)


def check_first_trial(log0, ref):
    # the damped solve in double precision: relative 1e-10 on the costs, the
    # damping and the gain ratio (the system's condition number is ~1e4)
    for key in ("chi_before", "chi_after", "lambda", "scale", "rho"):
        assert float(log0[key]) == pytest.approx(float(ref[key]), rel=1e-10), key


def test_oracle_first_lm_trial_matches_50_digit_values(kat):
    r = oracle.optimize(problem(kat["problem"]), 1)
    check_first_trial(r["log"][0], kat["lm_first_trial"])


@pytest.mark.gpu
def test_gpu_first_lm_trial_matches_50_digit_values(kat, gpu):
    from mcvslam_gb300 import ba

    with ba.Solver(precision="fp64", device=0) as s:
        s.load(problem(kat["problem"]))
        s.optimize(1)
        log = s.trial_log()
    check_first_trial(log[0], kat["lm_first_trial"])


@pytest.mark.gpu
def test_gpu_reprojection_matches_50_digit_values(kat, gpu):
    import torch

    from mcvslam_gb300 import autograd

    P = kat["problem"]
    pr = problem(P)
    qt = np.array([[float(v) for v in q] for q in kat["pose_qt"]])
    ext = np.stack([oracle.mat44f_to_qt(np.array(T, np.float32))[:7] for T in P["cam_Tcb"]])
    e = pr.edge_pose
    c = pr.edge_cam
    dev = torch.device("cuda:0")

    def t(a):
        return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device=dev)

    pose_qt, ext_qt = t(qt[e]), t(ext[c])
    X = t(pr.point_Xw.astype(np.float64)[pr.edge_point])
    K = t(pr.cam_K.astype(np.float64)[c])
    obs = t(pr.edge_obs.astype(np.float64)[:, :2])
    res = autograd.reprojection_residual(pose_qt, ext_qt, X, K, obs).cpu().numpy()
    Jp, _, Jx = (j.cpu().numpy() for j in autograd.jacobians(pose_qt, ext_qt, X, K))
    for i, ref in enumerate(kat["mono_edges"]):
        np.testing.assert_allclose(res[i], [float(v) for v in ref["e"]], rtol=1e-12, atol=1e-11)
        np.testing.assert_allclose(Jp[i], np.array(ref["J_pose"], dtype=np.float64), rtol=1e-12, atol=1e-10)
        np.testing.assert_allclose(Jx[i], np.array(ref["J_point"], dtype=np.float64), rtol=1e-12, atol=1e-10)
