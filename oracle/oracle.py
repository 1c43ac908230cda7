"""ctypes front end of the CPU oracle -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.

Only the tests, the smoke check and the benchmark's CPU legs import this
module; the product path never does.  Parity status: unpinned (the
reference has no golden vectors and cannot be built here); see the header
of g2o_oracle.cpp for what the restatement follows.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from oracle import build_oracle

_LIBS: dict = {}

c_float_p = ctypes.POINTER(ctypes.c_float)
c_double_p = ctypes.POINTER(ctypes.c_double)
c_u8_p = ctypes.POINTER(ctypes.c_uint8)
c_i32_p = ctypes.POINTER(ctypes.c_int32)


class OrcProblem(ctypes.Structure):
    _fields_ = [
        ("n_cams", ctypes.c_int32), ("cam_K", c_float_p), ("cam_bf", c_float_p), ("cam_Tcb", c_float_p),
        ("n_poses", ctypes.c_int32), ("pose_Tcw", c_float_p), ("pose_fixed", c_u8_p),
        ("n_points", ctypes.c_int32), ("point_Xw", c_float_p), ("point_fixed", c_u8_p),
        ("n_edges", ctypes.c_int32), ("edge_type", c_u8_p), ("edge_pose", c_i32_p),
        ("edge_point", c_i32_p), ("edge_cam", c_i32_p), ("edge_obs", c_float_p),
        ("edge_info", c_float_p), ("edge_delta", c_float_p), ("edge_robust", c_u8_p),
        ("edge_level", c_u8_p),
    ]


class OrcTrialLog(ctypes.Structure):
    _fields_ = [
        ("iteration", ctypes.c_int32), ("trial", ctypes.c_int32), ("chi_before", ctypes.c_double),
        ("chi_after", ctypes.c_double), ("lambda_", ctypes.c_double), ("scale", ctypes.c_double),
        ("rho", ctypes.c_double), ("accepted", ctypes.c_int32), ("solve_ok", ctypes.c_int32),
    ]


class OrcResult(ctypes.Structure):
    _fields_ = [
        ("pose_qt", c_double_p), ("pose_Tcw", c_float_p), ("point_X", c_double_p),
        ("edge_chi2", c_double_p), ("edge_level", c_u8_p), ("log", ctypes.POINTER(OrcTrialLog)),
        ("log_cap", ctypes.c_int32), ("n_log", ctypes.c_int32), ("iterations_done", ctypes.c_int32),
        ("n_active_edges", ctypes.c_int32), ("final_chi2", ctypes.c_double),
        ("seconds_linearize", ctypes.c_double), ("seconds_total", ctypes.c_double),
        ("edges_linearized", ctypes.c_int64),
    ]


LOG_DTYPE = np.dtype([("iteration", np.int32), ("trial", np.int32), ("chi_before", np.float64),
                      ("chi_after", np.float64), ("lambda", np.float64), ("scale", np.float64),
                      ("rho", np.float64), ("accepted", np.int32), ("solve_ok", np.int32)], align=True)


def lib(threads: bool = False):
    name = "liboracle_omp.so" if threads else "liboracle.so"
    if name not in _LIBS:
        paths = build_oracle.build()
        L = ctypes.CDLL(paths[name])
        L.orc_optimize.argtypes = [ctypes.POINTER(OrcProblem), ctypes.c_int, ctypes.c_int, ctypes.POINTER(OrcResult)]
        L.orc_pose_optimization.argtypes = [ctypes.POINTER(OrcProblem), ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                            ctypes.c_int, ctypes.c_int, ctypes.POINTER(OrcResult),
                                            ctypes.POINTER(ctypes.c_int)]
        L.orc_local_ba.argtypes = [ctypes.POINTER(OrcProblem), ctypes.c_int, ctypes.c_float, ctypes.c_int,
                                   ctypes.POINTER(OrcResult), ctypes.POINTER(ctypes.c_int)]
        L.orc_linearize_edges.argtypes = [ctypes.POINTER(OrcProblem), c_double_p, c_double_p, c_double_p]
        L.orc_normal_equations.argtypes = [ctypes.POINTER(OrcProblem), ctypes.c_double, c_double_p, c_double_p,
                                           c_double_p, ctypes.c_int]
        L.orc_knn_hamming.argtypes = [c_u8_p, ctypes.c_int32, c_u8_p, ctypes.c_int32, c_i32_p, c_i32_p, ctypes.c_float,
                                      ctypes.c_int32, c_u8_p, ctypes.c_int32]
        L.orc_knn_hamming.restype = None
        for fn in ("orc_se3_exp", "orc_mat44f_to_qt", "orc_qt_to_mat44f", "orc_huber", "orc_compose", "orc_map"):
            getattr(L, fn).restype = None
        _LIBS[name] = L
    return _LIBS[name]


def _ptr(a, t):
    return a.ctypes.data_as(t) if a is not None else None


def problem_struct(pr):
    """Pack a mcvslam_gb300.synth.Problem into the C struct; returns (struct, keepalive)."""
    keep = {}

    def arr(name, dt, shape_last=None):
        a = np.ascontiguousarray(getattr(pr, name), dtype=dt)
        keep[name] = a
        return a

    s = OrcProblem()
    s.n_cams = pr.n_cams
    s.cam_K = _ptr(arr("cam_K", np.float32), c_float_p)
    s.cam_bf = _ptr(arr("cam_bf", np.float32), c_float_p)
    s.cam_Tcb = _ptr(arr("cam_Tcb", np.float32), c_float_p)
    s.n_poses = pr.n_poses
    s.pose_Tcw = _ptr(arr("pose_Tcw", np.float32), c_float_p)
    s.pose_fixed = _ptr(arr("pose_fixed", np.uint8), c_u8_p)
    s.n_points = pr.n_points
    s.point_Xw = _ptr(arr("point_Xw", np.float32), c_float_p)
    s.point_fixed = _ptr(arr("point_fixed", np.uint8), c_u8_p)
    s.n_edges = pr.n_edges
    s.edge_type = _ptr(arr("edge_type", np.uint8), c_u8_p)
    s.edge_pose = _ptr(arr("edge_pose", np.int32), c_i32_p)
    s.edge_point = _ptr(arr("edge_point", np.int32), c_i32_p)
    s.edge_cam = _ptr(arr("edge_cam", np.int32), c_i32_p)
    s.edge_obs = _ptr(arr("edge_obs", np.float32), c_float_p)
    s.edge_info = _ptr(arr("edge_info", np.float32), c_float_p)
    s.edge_delta = _ptr(arr("edge_delta", np.float32), c_float_p)
    s.edge_robust = _ptr(arr("edge_robust", np.uint8), c_u8_p)
    s.edge_level = _ptr(arr("edge_level", np.uint8), c_u8_p)
    return s, keep


def _result(pr, log_cap):
    out = {
        "pose_qt": np.zeros((pr.n_poses, 7)),
        "pose_Tcw": np.zeros((pr.n_poses, 16), np.float32),
        "point_X": np.zeros((pr.n_points, 3)),
        "edge_chi2": np.zeros(pr.n_edges),
        "edge_level": np.zeros(pr.n_edges, np.uint8),
        "log": np.zeros(log_cap, LOG_DTYPE),
    }
    r = OrcResult()
    r.pose_qt = _ptr(out["pose_qt"], c_double_p)
    r.pose_Tcw = _ptr(out["pose_Tcw"], c_float_p)
    r.point_X = _ptr(out["point_X"], c_double_p)
    r.edge_chi2 = _ptr(out["edge_chi2"], c_double_p)
    r.edge_level = _ptr(out["edge_level"], c_u8_p)
    r.log = out["log"].ctypes.data_as(ctypes.POINTER(OrcTrialLog))
    r.log_cap = log_cap
    return r, out


def _finish(r, out):
    out["log"] = out["log"][: min(r.n_log, r.log_cap)].copy()
    out["iterations_done"] = r.iterations_done
    out["n_active_edges"] = r.n_active_edges
    out["final_chi2"] = r.final_chi2
    out["seconds_linearize"] = r.seconds_linearize
    out["seconds_total"] = r.seconds_total
    out["edges_linearized"] = r.edges_linearized
    return out


def optimize(pr, iterations: int, n_threads: int = 1, log_cap: int = 4096) -> dict:
    s, keep = problem_struct(pr)
    r, out = _result(pr, log_cap)
    ret = lib(n_threads > 1).orc_optimize(ctypes.byref(s), iterations, n_threads, ctypes.byref(r))
    out = _finish(r, out)
    out["ret"] = ret
    return out


def pose_optimization(pr, rounds: int = 4, iters: int = 15, chi2_thr: float = 5.991,
                      drop_robust_round: int = 2, n_threads: int = 1, log_cap: int = 4096) -> dict:
    s, keep = problem_struct(pr)
    r, out = _result(pr, log_cap)
    written = ctypes.c_int(0)
    ret = lib(n_threads > 1).orc_pose_optimization(ctypes.byref(s), rounds, iters, chi2_thr, drop_robust_round,
                                                   n_threads, ctypes.byref(r), ctypes.byref(written))
    out = _finish(r, out)
    out["ret"] = ret
    out["pose_written"] = written.value
    return out


def local_ba(pr, iterations: int = 10, chi2_thr: float = 5.991, n_threads: int = 1, log_cap: int = 4096) -> dict:
    s, keep = problem_struct(pr)
    r, out = _result(pr, log_cap)
    written = ctypes.c_int(0)
    ret = lib(n_threads > 1).orc_local_ba(ctypes.byref(s), iterations, chi2_thr, n_threads, ctypes.byref(r),
                                          ctypes.byref(written))
    out = _finish(r, out)
    out["ret"] = ret
    out["written"] = written.value
    return out


def linearize_edges(pr):
    s, keep = problem_struct(pr)
    E = pr.n_edges
    err = np.zeros((E, 3))
    Jl = np.zeros((E, 3, 3))
    Jp = np.zeros((E, 3, 6))
    lib().orc_linearize_edges(ctypes.byref(s), _ptr(err, c_double_p), _ptr(Jl, c_double_p), _ptr(Jp, c_double_p))
    return err, Jl, Jp


def normal_equations(pr, lam: float, cap: int = 4000):
    s, keep = problem_struct(pr)
    H = np.zeros(cap * cap)
    b = np.zeros(cap)
    x = np.zeros(cap)
    N = lib().orc_normal_equations(ctypes.byref(s), lam, _ptr(H, c_double_p), _ptr(b, c_double_p),
                                   _ptr(x, c_double_p), cap)
    if N <= 0:
        raise ValueError(f"normal equations too large or empty ({N})")
    return H[: N * N].reshape(N, N), b[:N], x[:N]


def se3_exp(u) -> np.ndarray:
    u = np.ascontiguousarray(u, np.float64)
    o = np.zeros(7)
    lib().orc_se3_exp(_ptr(u, c_double_p), _ptr(o, c_double_p))
    return o


def mat44f_to_qt(T) -> np.ndarray:
    T = np.ascontiguousarray(T, np.float32).reshape(16)
    o = np.zeros(7)
    lib().orc_mat44f_to_qt(_ptr(T, c_float_p), _ptr(o, c_double_p))
    return o


def qt_to_mat44f(qt) -> np.ndarray:
    qt = np.ascontiguousarray(qt, np.float64)
    o = np.zeros(16, np.float32)
    lib().orc_qt_to_mat44f(_ptr(qt, c_double_p), _ptr(o, c_float_p))
    return o.reshape(4, 4)


def huber(e2: float, delta: float) -> np.ndarray:
    o = np.zeros(3)
    lib().orc_huber(ctypes.c_double(e2), ctypes.c_double(delta), _ptr(o, c_double_p))
    return o


def compose(a, b) -> np.ndarray:
    a = np.ascontiguousarray(a, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    o = np.zeros(7)
    lib().orc_compose(_ptr(a, c_double_p), _ptr(b, c_double_p), _ptr(o, c_double_p))
    return o


def map_point(qt, X) -> np.ndarray:
    qt = np.ascontiguousarray(qt, np.float64)
    X = np.ascontiguousarray(X, np.float64)
    o = np.zeros(3)
    lib().orc_map(_ptr(qt, c_double_p), _ptr(X, c_double_p), _ptr(o, c_double_p))
    return o


def knn_hamming(query, train, ratio: float = 0.6, max_dist: int = 46, n_threads: int = 1):
    """Matcher::KnnMatch (k = 2) over 32-byte descriptors: [nq, 2] train
    indices and distances plus the FilterRatio/FilterThreshold keep flag."""
    q = np.ascontiguousarray(query, np.uint8).reshape(-1, 32)
    t = np.ascontiguousarray(train, np.uint8).reshape(-1, 32)
    nq, nt = q.shape[0], t.shape[0]
    idx = np.zeros((nq, 2), np.int32)
    dist = np.zeros((nq, 2), np.int32)
    keep = np.zeros(nq, np.uint8)
    lib(n_threads > 1).orc_knn_hamming(_ptr(q, c_u8_p), nq, _ptr(t, c_u8_p), nt, _ptr(idx, c_i32_p),
                                        _ptr(dist, c_i32_p), ratio, max_dist, _ptr(keep, c_u8_p), n_threads)
    return idx, dist, keep


def project_match(b, n_threads: int = 1):
    """Object::ProjectBunchMapPoints over a synth.ProjectionBatch: (kp_bind
    after the call, mp_match, obj_count)."""
    L = lib(n_threads > 1)
    c_f, c_i, c_u8 = c_float_p, c_i32_p, c_u8_p
    if not hasattr(L, "_pm_sig"):
        L.orc_project_match.argtypes = [ctypes.c_int32, ctypes.c_int32, c_f, c_f, c_i, c_f, c_f, ctypes.c_int32, ctypes.c_float,
                                        ctypes.c_int32, c_i, c_f, c_u8, c_i, c_f, c_u8, c_i, c_i, c_i, c_i, c_i]
        L.orc_project_match.restype = None
        L._pm_sig = True
    a = lambda x, dt: np.ascontiguousarray(x, dt)  # noqa: E731
    keep = [a(b.obj_Rt, np.float32), a(b.obj_K, np.float32), a(b.obj_size, np.int32), a(b.obj_radius, np.float32),
            a(b.obj_scale, np.float32), a(b.kp_begin, np.int32), a(b.kp_xy, np.float32), a(b.kp_desc, np.uint8),
            a(b.mp_begin, np.int32), a(b.mp_X, np.float32), a(b.mp_desc, np.uint8), a(b.mp_level, np.int32),
            a(b.mp_id, np.int32)]
    kp_bind = np.array(b.kp_bind, np.int32, copy=True)
    nm = int(b.mp_begin[-1])
    mp_match = np.zeros(nm, np.int32)
    obj_count = np.zeros(b.n_objects, np.int32)
    ts = [c_f, c_f, c_i, c_f, c_f, c_i, c_f, c_u8, c_i, c_f, c_u8, c_i, c_i]
    p = [_ptr(x, t) for x, t in zip(keep, ts)]
    L.orc_project_match(n_threads, b.n_objects, p[0], p[1], p[2], p[3], p[4], int(b.obj_scale.shape[1]), b.ratio, b.max_dist,
                        p[5], p[6], p[7], p[8], p[9], p[10], p[11], p[12], _ptr(kp_bind, c_i), _ptr(mp_match, c_i),
                        _ptr(obj_count, c_i))
    return kp_bind, mp_match, obj_count


def stereo_match(sb, n_threads: int = 1):
    """Frame::ComputeStereoMatch over a synth.StereoBatch: (u_right, depth) per left keypoint."""
    L = lib(n_threads > 1)
    c_f, c_i, c_u8 = c_float_p, c_i32_p, c_u8_p
    c_i64 = ctypes.POINTER(ctypes.c_int64)
    if not hasattr(L, "_sm_sig"):
        i32 = ctypes.c_int32
        L.orc_stereo_match.argtypes = [i32, i32, i32, c_f, c_f, c_i, c_i, c_i64, ctypes.c_int64, c_u8, c_u8, i32,
                                       ctypes.c_float, ctypes.c_float, c_i, c_f, c_i, c_u8, c_i, c_f, c_i, c_u8,
                                       c_f, c_f]
        L.orc_stereo_match.restype = None
        L._sm_sig = True
    a = lambda x, dt: np.ascontiguousarray(x, dt)  # noqa: E731
    k = dict(scale=a(sb.scale, np.float32), inv=a(sb.inv_scale, np.float32), lr=a(sb.level_rows, np.int32),
             lc=a(sb.level_cols, np.int32), off=a(sb.level_offset, np.int64), lp=a(sb.left_pyr, np.uint8),
             rp=a(sb.right_pyr, np.uint8), lb=a(sb.left_begin, np.int32), lxy=a(sb.left_xy, np.float32),
             lo=a(sb.left_oct, np.int32), ld=a(sb.left_desc, np.uint8), rb=a(sb.right_begin, np.int32),
             rxy=a(sb.right_xy, np.float32), ro=a(sb.right_oct, np.int32), rd=a(sb.right_desc, np.uint8))
    nl = int(sb.left_begin[-1])
    u = np.zeros(nl, np.float32)
    d = np.zeros(nl, np.float32)
    L.orc_stereo_match(n_threads, sb.n_frames, int(sb.scale.shape[0]), _ptr(k["scale"], c_f), _ptr(k["inv"], c_f),
                       _ptr(k["lr"], c_i), _ptr(k["lc"], c_i), _ptr(k["off"], c_i64), int(sb.pyr_bytes),
                       _ptr(k["lp"], c_u8), _ptr(k["rp"], c_u8), int(sb.image_rows), float(sb.b), float(sb.bf),
                       _ptr(k["lb"], c_i), _ptr(k["lxy"], c_f), _ptr(k["lo"], c_i), _ptr(k["ld"], c_u8),
                       _ptr(k["rb"], c_i), _ptr(k["rxy"], c_f), _ptr(k["ro"], c_i), _ptr(k["rd"], c_u8),
                       _ptr(u, c_f), _ptr(d, c_f))
    return u, d


class OrcMap(ctypes.Structure):
    _fields_ = [
        ("n_keyframes", ctypes.c_int32), ("kf_id", ctypes.POINTER(ctypes.c_int64)), ("obs_begin", c_i32_p),
        ("obs_point", c_i32_p), ("obs_object", c_u8_p), ("obs_uv", c_float_p), ("obs_ur", c_float_p),
        ("obs_octave", c_u8_p), ("n_points", ctypes.c_int32), ("mp_kf_begin", c_i32_p), ("mp_kf", c_i32_p),
        ("ess_begin", c_i32_p), ("ess_adj", c_i32_p), ("inv_sigma2_left", c_float_p),
        ("inv_sigma2_wide", c_float_p),
    ]


class OrcWindowOut(ctypes.Structure):
    _fields_ = [
        ("kf_role", c_u8_p), ("pose_kf", c_i32_p), ("pose_fixed", c_u8_p), ("point_mp", c_i32_p),
        ("point_fixed", c_u8_p), ("max_edges", ctypes.c_int32), ("edge_type", c_u8_p), ("edge_pose", c_i32_p),
        ("edge_point", c_i32_p), ("edge_cam", c_i32_p), ("edge_obs", c_float_p), ("edge_info", c_float_p),
        ("edge_delta", c_float_p), ("n_local", ctypes.c_int32), ("n_anchor", ctypes.c_int32),
        ("n_poses", ctypes.c_int32), ("n_points", ctypes.c_int32), ("n_edges", ctypes.c_int32),
    ]


def local_window(m, cur: int, hop: int = 1) -> dict:
    """Map::AddKeyFrame's local-BA set-up on a synth.MapTables: the window
    (kf_role bit 0 optimised, bit 1 anchor), the problem's vertices in
    BAoptimizer insertion order and its edges (window_oracle.cpp)."""
    L = lib(False)
    if not hasattr(L, "_win_sig"):
        L.orc_local_window.argtypes = [ctypes.POINTER(OrcMap), ctypes.c_int32, ctypes.c_int32,
                                       ctypes.POINTER(OrcWindowOut)]
        L._win_sig = True
    a = lambda x, dt: np.ascontiguousarray(x, dt)  # noqa: E731
    k = dict(id=a(m.kf_id, np.int64), ob=a(m.obs_begin, np.int32), op=a(m.obs_point, np.int32),
             oo=a(m.obs_object, np.uint8), uv=a(m.obs_uv, np.float32), ur=a(m.obs_ur, np.float32),
             oc=a(m.obs_octave, np.uint8), mb=a(m.mp_kf_begin, np.int32), mk=a(m.mp_kf, np.int32),
             eb=a(m.ess_begin, np.int32), ea=a(m.ess_adj, np.int32), sl=a(m.inv_sigma2_left, np.float32),
             sw=a(m.inv_sigma2_wide, np.float32))
    s = OrcMap(m.n_keyframes, k["id"].ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), _ptr(k["ob"], c_i32_p),
               _ptr(k["op"], c_i32_p), _ptr(k["oo"], c_u8_p), _ptr(k["uv"], c_float_p), _ptr(k["ur"], c_float_p),
               _ptr(k["oc"], c_u8_p), m.n_points, _ptr(k["mb"], c_i32_p), _ptr(k["mk"], c_i32_p),
               _ptr(k["eb"], c_i32_p), _ptr(k["ea"], c_i32_p), _ptr(k["sl"], c_float_p), _ptr(k["sw"], c_float_p))
    nk, cap = m.n_keyframes, 2 * len(m.obs_point) + 1  # a keyframe can be anchor and member
    o = dict(kf_role=np.zeros(nk, np.uint8), pose_kf=np.zeros(nk, np.int32), pose_fixed=np.zeros(nk, np.uint8),
             point_mp=np.zeros(m.n_points, np.int32), point_fixed=np.zeros(m.n_points, np.uint8),
             edge_type=np.zeros(cap, np.uint8), edge_pose=np.zeros(cap, np.int32), edge_point=np.zeros(cap, np.int32),
             edge_cam=np.zeros(cap, np.int32), edge_obs=np.zeros((cap, 3), np.float32),
             edge_info=np.zeros(cap, np.float32), edge_delta=np.zeros(cap, np.float32))
    w = OrcWindowOut(_ptr(o["kf_role"], c_u8_p), _ptr(o["pose_kf"], c_i32_p), _ptr(o["pose_fixed"], c_u8_p),
                     _ptr(o["point_mp"], c_i32_p), _ptr(o["point_fixed"], c_u8_p), cap,
                     _ptr(o["edge_type"], c_u8_p), _ptr(o["edge_pose"], c_i32_p), _ptr(o["edge_point"], c_i32_p),
                     _ptr(o["edge_cam"], c_i32_p), _ptr(o["edge_obs"], c_float_p), _ptr(o["edge_info"], c_float_p),
                     _ptr(o["edge_delta"], c_float_p), 0, 0, 0, 0, 0)
    rc = L.orc_local_window(ctypes.byref(s), cur, hop, ctypes.byref(w))
    if rc != 0:
        raise RuntimeError(f"orc_local_window returned {rc}")
    npo, npt, ne = w.n_poses, w.n_points, w.n_edges
    for key in ("pose_kf", "pose_fixed"):
        o[key] = o[key][:npo]
    for key in ("point_mp", "point_fixed"):
        o[key] = o[key][:npt]
    for key in ("edge_type", "edge_pose", "edge_point", "edge_cam", "edge_obs", "edge_info", "edge_delta"):
        o[key] = o[key][:ne]
    o.update(n_local=w.n_local, n_anchor=w.n_anchor)
    return o


def window_problem(m, w: dict):
    """The assembled window as a synth.Problem (camera 0 LEFT with
    T_cam_body = I and the stereo bf, camera 1 WIDE), for the oracle solver."""
    from mcvslam_gb300 import synth

    E = len(w["edge_type"])
    return synth.Problem(
        cam_K=np.stack([m.K_left, m.K_wide]).astype(np.float32), cam_bf=np.array([m.bf, 0.0], np.float32),
        cam_Tcb=np.stack([np.eye(4, dtype=np.float32).reshape(16), m.T_wide_body]).astype(np.float32),
        cam_size=np.array([[512, 512], [512, 512]], np.int32),
        pose_Tcw=m.kf_Tcw[w["pose_kf"]].astype(np.float32), pose_fixed=w["pose_fixed"].astype(np.uint8),
        point_Xw=m.mp_Xw[w["point_mp"]].astype(np.float32), point_fixed=w["point_fixed"].astype(np.uint8),
        edge_type=w["edge_type"], edge_pose=w["edge_pose"], edge_point=w["edge_point"], edge_cam=w["edge_cam"],
        edge_obs=w["edge_obs"], edge_info=w["edge_info"], edge_delta=w["edge_delta"],
        edge_robust=np.ones(E, np.uint8), edge_level=np.zeros(E, np.uint8), name="local_window")
