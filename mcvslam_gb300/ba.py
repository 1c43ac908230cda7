"""Host-side mirror of MCVSLAM's BAoptimizer / PoseEstimation interface.

``Solver`` wraps one ``mcba_problem`` handle of libmcba.so (bulk loading,
optimisation, read-back).  ``BAoptimizer`` keeps the reference's method names
(include/BAoptimizer.hpp:29-80) so that code written against the reference
reads the same; ``KeyFrame``/``MapPoint`` are the minimal stand-ins for the
fields those methods touch (pose, cameras, rig extrinsic, stereo baseline,
per-level inverse sigma^2, world position).
"""
from __future__ import annotations

import ctypes
import dataclasses
from typing import Callable, Dict, List, Optional, Tuple

import numpy as np

from mcvslam_gb300 import _native as N
from mcvslam_gb300 import synth

PRECISIONS = {"fp64": 0, "plain": 0, "mixed": 1}

LOG_DTYPE = np.dtype([("iteration", np.int32), ("trial", np.int32), ("chi_before", np.float64),
                      ("chi_after", np.float64), ("lambda", np.float64), ("scale", np.float64),
                      ("rho", np.float64), ("accepted", np.int32), ("solve_ok", np.int32)], align=True)


def _p(a, t):
    return a.ctypes.data_as(t) if a is not None else None


class Solver:
    """One bundle-adjustment problem on the GPU."""

    def __init__(self, precision: str = "fp64", device: int = 0, use_graph: bool = True, tau: float = 1e-5,
                 max_trials: int = 10, stream: int = 0, profile: bool = False, host_structure: bool = False):
        self.L = N.lib()
        o = N.Options()
        self.L.mcba_default_options(ctypes.byref(o))
        o.precision = PRECISIONS[precision]
        o.device = device
        o.use_graph = 1 if use_graph else 0
        o.tau = tau
        o.max_trials = max_trials
        o.profile = 1 if profile else 0
        o.stream = stream or None
        o.host_structure = 1 if host_structure else 0
        h = ctypes.c_void_p()
        N.check(self.L.mcba_create(ctypes.byref(o), ctypes.byref(h)))
        self.h = h
        self.precision = precision
        self.n_poses = 0
        self.n_points = 0
        self.n_edges = 0

    # -- life cycle
    def close(self):
        if getattr(self, "h", None):
            self.L.mcba_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- graph
    _LOAD_ARRAYS = (("cam_K", np.float32), ("cam_bf", np.float32), ("cam_Tcb", np.float32),
                    ("pose_Tcw", np.float32), ("pose_fixed", np.uint8), ("point_Xw", np.float32),
                    ("point_fixed", np.uint8), ("edge_type", np.uint8), ("edge_pose", np.int32),
                    ("edge_point", np.int32), ("edge_cam", np.int32), ("edge_obs", np.float32),
                    ("edge_info", np.float32), ("edge_delta", np.float32), ("edge_robust", np.uint8),
                    ("edge_level", np.uint8))

    def load(self, pr: synth.Problem) -> "Solver":
        d = N.ProblemDesc()
        d.n_cams, d.n_poses, d.n_points, d.n_edges = pr.n_cams, pr.n_poses, pr.n_points, pr.n_edges
        keep = []  # converted copies live until mcba_load has copied them
        for name, dt in self._LOAD_ARRAYS:
            a = getattr(pr, name)
            if a.dtype != dt or not a.flags["C_CONTIGUOUS"]:
                a = np.ascontiguousarray(a, dtype=dt)
            keep.append(a)
            setattr(d, name, a.ctypes.data if a.size else None)
        N.check(self.L.mcba_load(self.h, ctypes.byref(d)), self.h)
        self.n_poses, self.n_points, self.n_edges = pr.n_poses, pr.n_points, pr.n_edges
        return self

    # -- solve
    def optimize(self, iterations: int) -> dict:
        st = N.Stats()
        r = self.L.mcba_optimize(self.h, iterations, ctypes.byref(st))
        if r not in (N.MCBA_OK, 2):
            N.check(r, self.h)
        d = st.as_dict()
        d["ret"] = r
        return d

    def prepare(self) -> None:
        N.check(self.L.mcba_prepare(self.h), self.h)

    def solve_prepared(self, iterations: int) -> dict:
        st = N.Stats()
        N.check(self.L.mcba_solve_prepared(self.h, iterations, ctypes.byref(st)), self.h)
        return st.as_dict()

    def fetch_state(self) -> None:
        N.check(self.L.mcba_fetch_state(self.h), self.h)

    def trial_log(self) -> np.ndarray:
        n = ctypes.c_int32(0)
        self.L.mcba_trial_log_get(self.h, None, 0, ctypes.byref(n))
        out = np.zeros(n.value, LOG_DTYPE)
        if n.value:
            N.check(self.L.mcba_trial_log_get(self.h, out.ctypes.data_as(ctypes.POINTER(N.TrialLog)), n.value,
                                              ctypes.byref(n)))
        return out

    def state(self) -> Tuple[np.ndarray, np.ndarray]:
        qt = np.zeros((self.n_poses, 7))
        X = np.zeros((self.n_points, 3))
        N.check(self.L.mcba_get_state(self.h, _p(qt, N.c_double_p), _p(X, N.c_double_p)), self.h)
        return qt, X

    def set_state(self, qt=None, X=None) -> None:
        qt = None if qt is None else np.ascontiguousarray(qt, np.float64)
        X = None if X is None else np.ascontiguousarray(X, np.float64)
        N.check(self.L.mcba_set_state(self.h, _p(qt, N.c_double_p), _p(X, N.c_double_p)), self.h)

    def keyframe(self, i: int) -> np.ndarray:
        T = np.zeros(16, np.float32)
        N.check(self.L.mcba_get_keyframe(self.h, i, _p(T, N.c_float_p)), self.h)
        return T.reshape(4, 4)

    def mappoint(self, i: int) -> np.ndarray:
        X = np.zeros(3, np.float32)
        N.check(self.L.mcba_get_mappoint(self.h, i, _p(X, N.c_float_p)), self.h)
        return X

    def edge_chi2(self) -> np.ndarray:
        out = np.zeros(self.n_edges)
        N.check(self.L.mcba_edge_chi2(self.h, _p(out, N.c_double_p)), self.h)
        return out

    def levels(self) -> np.ndarray:
        out = np.zeros(self.n_edges, np.uint8)
        N.check(self.L.mcba_get_edge_levels(self.h, _p(out, N.c_u8_p)), self.h)
        return out

    def set_levels(self, lv) -> None:
        lv = np.ascontiguousarray(lv, np.uint8)
        N.check(self.L.mcba_set_edge_levels(self.h, _p(lv, N.c_u8_p)), self.h)

    def set_robust(self, rb) -> None:
        rb = np.ascontiguousarray(rb, np.uint8)
        N.check(self.L.mcba_set_edge_robust(self.h, _p(rb, N.c_u8_p)), self.h)

    def pose_optimization(self, rounds=4, iterations=15, chi2_thr=5.991, drop_robust_round=2) -> Tuple[int, int]:
        a, b = ctypes.c_int32(0), ctypes.c_int32(0)
        N.check(self.L.mcba_pose_optimization(self.h, rounds, iterations, chi2_thr, drop_robust_round,
                                              ctypes.byref(a), ctypes.byref(b)), self.h)
        return a.value, b.value

    def local_ba(self, iterations=10, chi2_thr=5.991) -> Tuple[int, int]:
        a, b = ctypes.c_int32(0), ctypes.c_int32(0)
        N.check(self.L.mcba_local_ba(self.h, iterations, chi2_thr, ctypes.byref(a), ctypes.byref(b)), self.h)
        return a.value, b.value

    def local_window(self, m, cur: int, hop: int = 1) -> dict:
        """Map::AddKeyFrame's local-BA set-up for keyframe `cur` of the map
        tables `m` (a synth.MapTables) on the GPU: the window is chosen and its
        problem loaded into this solver (mcba_local_window).  Returns the roles
        (bit 0 optimised, bit 1 anchor), the map keyframe of each pose, the map
        point of each point, ThisMapPointBeFix per point and the counts."""
        a = {}

        def arr(name, dt):
            x = np.ascontiguousarray(getattr(m, name), dtype=dt)
            a[name] = x
            return x.ctypes.data

        d = N.MapDesc()
        d.n_keyframes = m.n_keyframes
        d.kf_id = arr("kf_id", np.int64)
        d.kf_Tcw = arr("kf_Tcw", np.float32)
        d.obs_begin = arr("obs_begin", np.int32)
        d.obs_point = arr("obs_point", np.int32)
        d.obs_object = arr("obs_object", np.uint8)
        d.obs_uv = arr("obs_uv", np.float32)
        d.obs_ur = arr("obs_ur", np.float32)
        d.obs_octave = arr("obs_octave", np.uint8)
        d.n_points = m.n_points
        d.mp_Xw = arr("mp_Xw", np.float32)
        d.mp_kf_begin = arr("mp_kf_begin", np.int32)
        d.mp_kf = arr("mp_kf", np.int32)
        d.ess_begin = arr("ess_begin", np.int32)
        d.ess_adj = arr("ess_adj", np.int32)
        d.n_levels = int(len(m.inv_sigma2_left))
        d.inv_sigma2_left = arr("inv_sigma2_left", np.float32)
        d.inv_sigma2_wide = arr("inv_sigma2_wide", np.float32)
        d.K_left[:] = [float(x) for x in m.K_left]
        d.K_wide[:] = [float(x) for x in m.K_wide]
        d.T_wide_body[:] = [float(x) for x in np.asarray(m.T_wide_body).reshape(16)]
        d.bf = float(m.bf)
        role = np.zeros(m.n_keyframes, np.uint8)
        pose_kf = np.zeros(m.n_keyframes, np.int32)
        point_mp = np.zeros(max(m.n_points, 1), np.int32)
        point_fixed = np.zeros(max(m.n_points, 1), np.uint8)
        info = N.WindowInfo()
        N.check(self.L.mcba_local_window(self.h, ctypes.byref(d), cur, hop, _p(role, N.c_u8_p),
                                         _p(pose_kf, N.c_i32_p), _p(point_mp, N.c_i32_p), _p(point_fixed, N.c_u8_p),
                                         ctypes.byref(info)), self.h)
        self.n_poses, self.n_points, self.n_edges = info.n_poses, info.n_points, info.n_edges
        return {"kf_role": role, "pose_kf": pose_kf[:info.n_poses], "point_mp": point_mp[:info.n_points],
                "point_fixed": point_fixed[:info.n_points], "n_local": info.n_local, "n_anchor": info.n_anchor,
                "n_fixed_points": info.n_fixed_points, "n_edges": info.n_edges}

    def dump_hessian(self, path: str) -> None:
        N.check(self.L.mcba_dump_hessian(self.h, path.encode()), self.h)


def batch_pose_only(problems, precision: str = "mixed", rounds: int = 4, iterations: int = 15,
                    chi2_thr: float = 5.991, drop_robust_round: int = 2, device: int = 0) -> dict:
    """PoseOptimization of many single-frame problems in one device pass.

    Each problem is a synth.Problem with one keyframe and fixed points (as
    produced by synth.pose_only); all problems share the rig of the first.
    Returns the FP64 poses (x y z w tx ty tz), per-problem inlier counts, the
    per-edge outlier levels (concatenated in problem order) and the device time."""
    n = len(problems)
    counts = np.array([p.n_edges for p in problems], np.int32)
    edge_begin = np.zeros(n + 1, np.int32)
    np.cumsum(counts, out=edge_begin[1:])
    rig = problems[0]
    # float 4x4 T_body_world -> FP64 quaternion + translation with the library's
    # own conversion (Converter::toSE3Quat)
    conv = Solver()
    for p in problems:
        T = np.ascontiguousarray(p.pose_Tcw[0], np.float32)
        N.check(conv.L.mcba_add_keyframe(conv.h, _p(T, N.c_float_p), 0, None), conv.h)
    conv.n_poses = n
    qt = np.ascontiguousarray(conv.state()[0])
    conv.close()
    cam = np.ascontiguousarray(np.concatenate([p.edge_cam for p in problems]).astype(np.int32))
    obs = np.ascontiguousarray(np.concatenate([p.edge_obs[:, :2] for p in problems]).astype(np.float32))
    Xw = np.ascontiguousarray(np.concatenate([p.point_Xw[p.edge_point] for p in problems]).astype(np.float32))
    info = np.ascontiguousarray(np.concatenate([p.edge_info for p in problems]).astype(np.float32))
    delta = np.ascontiguousarray(np.concatenate([p.edge_delta for p in problems]).astype(np.float32))
    level = np.zeros(int(edge_begin[-1]), np.uint8)
    inliers = np.zeros(n, np.int32)
    ms = ctypes.c_double(0.0)
    K = np.ascontiguousarray(rig.cam_K, np.float32)
    Tcb = np.ascontiguousarray(rig.cam_Tcb, np.float32)
    L = N.lib()
    N.check(L.mcba_batch_pose_only(device, PRECISIONS[precision], n, _p(edge_begin, N.c_i32_p), rig.n_cams,
                                   _p(K, N.c_float_p), _p(Tcb, N.c_float_p), _p(cam, N.c_i32_p),
                                   _p(obs, N.c_float_p), _p(Xw, N.c_float_p), _p(info, N.c_float_p),
                                   _p(delta, N.c_float_p), rounds, iterations, chi2_thr, drop_robust_round,
                                   _p(qt, N.c_double_p), _p(level, N.c_u8_p), _p(inliers, N.c_i32_p),
                                   ctypes.byref(ms)))
    return {"pose_qt": qt, "inliers": inliers, "edge_level": level, "edge_begin": edge_begin,
            "ms_device": ms.value}


class LocalBABatch:
    """Many local-BA windows solved together (mcba_batch_*): as branches of one
    CUDA graph, or (persistent=True) in one persistent launch whose clusters
    take the windows from a device work queue."""

    def __init__(self, problems, precision: str = "mixed", device: int = 0):
        self.solvers = [Solver(precision=precision, device=device).load(pr) for pr in problems]
        self.L = N.lib()
        arr = (ctypes.c_void_p * len(self.solvers))(*[s.h.value for s in self.solvers])
        self._arr = arr
        N.check(self.L.mcba_batch_prepare(arr, len(self.solvers)))

    def solve(self, iterations: int = 10, persistent: bool = False, cluster_ctas: int = 0):
        """cluster_ctas (persistent launch only): 0 lets the autotuner choose
        the CTAs per window, 4 / 8 / 16 forces that size."""
        n = len(self.solvers)
        stats = (N.Stats * n)()
        ms = ctypes.c_double(0.0)
        if persistent:
            ctas = ctypes.c_int32(cluster_ctas)
            N.check(self.L.mcba_batch_solve_persistent(self._arr, n, iterations, stats, ctypes.byref(ms),
                                                       ctypes.byref(ctas)), self.solvers[0].h)
            self.cluster_ctas = ctas.value
        else:
            N.check(self.L.mcba_batch_solve(self._arr, n, iterations, stats, ctypes.byref(ms)), self.solvers[0].h)
        return [st.as_dict() for st in stats], ms.value

    def states(self):
        out = []
        for s in self.solvers:
            s.fetch_state()
            out.append(s.state())
        return out

    def close(self):
        for s in self.solvers:
            s.close()
        self.solvers = []

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def solve(pr: synth.Problem, iterations: int = 10, precision: str = "fp64", **kw) -> dict:
    """Load, optimise and read back one problem; returns stats, state and trial log."""
    with Solver(precision=precision, **kw) as s:
        s.load(pr)
        st = s.optimize(iterations)
        qt, X = s.state()
        return {"stats": st, "pose_qt": qt, "point_X": X, "log": s.trial_log()}


# ------------------------------------------------ reference-shaped facade --
@dataclasses.dataclass
class Camera:
    K: Tuple[float, float, float, float]   # fx fy cx cy (BaseCamera::parameters)


@dataclasses.dataclass
class KeyFrame:
    """The fields of MCVSLAM's Frame that BAoptimizer reads."""
    id: int
    Tcw: np.ndarray                          # float 4x4 T_body_world (GetPose)
    left: Camera
    wide: Camera
    Twl: np.ndarray                          # float 4x4 used as T_cam_body of the wide edges
    bf: float = 0.0
    inv_level_sigma2_left: Tuple[float, ...] = (1.0,)
    inv_level_sigma2_wide: Tuple[float, ...] = (1.0,)


@dataclasses.dataclass
class MapPoint:
    pos: np.ndarray                          # float[3] (GetWorldPos)

    def __hash__(self):
        return id(self)


class Edge:
    """The handful of g2o edge calls the reference's filter callbacks use."""

    def __init__(self, opt: "BAoptimizer", idx: int):
        self.opt, self.idx = opt, idx

    def level(self) -> int:
        return int(self.opt._levels[self.idx])

    def setLevel(self, lv: int) -> None:
        self.opt._levels[self.idx] = lv
        self.opt._dirty_levels = True

    def computeError(self) -> None:
        self.opt._refresh_chi2()

    def chi2(self) -> float:
        return float(self.opt._chi2[self.idx])

    def setRobustKernel(self, k) -> None:
        self.opt._robust[self.idx] = 0 if k is None or k == 0 else 1
        self.opt._dirty_robust = True


class BAoptimizer:
    """MCVSLAM::BAoptimizer on libmcba (include/BAoptimizer.hpp:29-80)."""

    thHuber2D = float(np.float32(np.sqrt(5.99)))
    thHuber3D = float(np.float32(np.sqrt(7.815)))

    def __init__(self, precision: str = "fp64", device: int = 0):
        self.s = Solver(precision=precision, device=device)
        self.L, self.h = self.s.L, self.s.h
        self.KF2ID: Dict[int, int] = {}
        self.MP2ID: Dict[int, int] = {}
        self.ALLKFS: Dict[int, KeyFrame] = {}
        self.ALLMPS: Dict[int, MapPoint] = {}
        self.EdgeInfos: Dict[Edge, Tuple[MapPoint, str]] = {}
        self._cams: Dict[tuple, int] = {}
        self._levels = np.zeros(0, np.uint8)
        self._robust = np.zeros(0, np.uint8)
        self._chi2 = np.zeros(0)
        self._dirty_levels = self._dirty_robust = False

    def _camera(self, K, Tcb) -> int:
        key = (tuple(np.float32(K)), np.asarray(Tcb, np.float32).tobytes())
        if key not in self._cams:
            Kf = np.ascontiguousarray(K, np.float32)
            T = np.ascontiguousarray(Tcb, np.float32).reshape(16)
            cid = ctypes.c_int32()
            N.check(self.L.mcba_add_camera(self.h, _p(Kf, N.c_float_p), 0.0, _p(T, N.c_float_p), ctypes.byref(cid)),
                    self.h)
            self._cams[key] = cid.value
        return self._cams[key]

    # src/BAoptimizer.cpp:22-31
    def addKeyFrame(self, kf: KeyFrame, fixed: bool = False) -> None:
        if id(kf) in self.KF2ID:
            return
        T = np.ascontiguousarray(kf.Tcw, np.float32).reshape(16)
        vid = ctypes.c_int32()
        N.check(self.L.mcba_add_keyframe(self.h, _p(T, N.c_float_p), 1 if (fixed or kf.id == 0) else 0,
                                         ctypes.byref(vid)), self.h)
        self.KF2ID[id(kf)] = vid.value
        self.ALLKFS[id(kf)] = kf
        self.s.n_poses += 1

    # src/BAoptimizer.cpp:33-42
    def addMapppint(self, mp: MapPoint, fixed: bool = False) -> None:
        if id(mp) in self.MP2ID:
            return
        X = np.ascontiguousarray(mp.pos, np.float32)
        vid = ctypes.c_int32()
        N.check(self.L.mcba_add_mappoint(self.h, _p(X, N.c_float_p), 1 if fixed else 0, ctypes.byref(vid)), self.h)
        self.MP2ID[id(mp)] = vid.value
        self.ALLMPS[id(mp)] = mp
        self.s.n_points += 1

    def _push(self, mp, obj):
        e = Edge(self, self.s.n_edges)
        self.s.n_edges += 1
        self._levels = np.append(self._levels, np.uint8(0))
        self._robust = np.append(self._robust, np.uint8(1))
        self.EdgeInfos[e] = (mp, obj)
        return e

    # src/BAoptimizer.cpp:45-65
    def addEdge(self, kf: KeyFrame, mp: MapPoint, uv, level: int) -> Edge:
        cam = self._camera(kf.left.K, np.eye(4))
        eid = ctypes.c_int32()
        N.check(self.L.mcba_add_edge_mono(self.h, self.KF2ID[id(kf)], self.MP2ID[id(mp)], cam, float(uv[0]),
                                          float(uv[1]), float(kf.inv_level_sigma2_left[level]), self.thHuber2D,
                                          ctypes.byref(eid)), self.h)
        return self._push(mp, "LEFT")

    # src/BAoptimizer.cpp:67-88
    def addEdgeStereo(self, kf: KeyFrame, mp: MapPoint, uv, ru: float, level: int) -> Edge:
        key = (tuple(np.float32(kf.left.K)), np.eye(4, dtype=np.float32).tobytes(), "stereo", float(kf.bf))
        if key not in self._cams:
            Kf = np.ascontiguousarray(kf.left.K, np.float32)
            T = np.eye(4, dtype=np.float32).reshape(16)
            cid = ctypes.c_int32()
            N.check(self.L.mcba_add_camera(self.h, _p(Kf, N.c_float_p), float(kf.bf), _p(T, N.c_float_p),
                                           ctypes.byref(cid)), self.h)
            self._cams[key] = cid.value
        eid = ctypes.c_int32()
        N.check(self.L.mcba_add_edge_stereo(self.h, self.KF2ID[id(kf)], self.MP2ID[id(mp)], self._cams[key],
                                            float(uv[0]), float(uv[1]), float(ru),
                                            float(kf.inv_level_sigma2_left[level]), self.thHuber3D,
                                            ctypes.byref(eid)), self.h)
        return self._push(mp, "LEFT")

    # src/BAoptimizer.cpp:90-108
    def addEdgeToBody(self, kf: KeyFrame, mp: MapPoint, uv, level: int) -> Edge:
        cam = self._camera(kf.wide.K, kf.Twl)
        eid = ctypes.c_int32()
        N.check(self.L.mcba_add_edge_mono(self.h, self.KF2ID[id(kf)], self.MP2ID[id(mp)], cam, float(uv[0]),
                                          float(uv[1]), float(kf.inv_level_sigma2_wide[level]), self.thHuber3D,
                                          ctypes.byref(eid)), self.h)
        return self._push(mp, "LEFT")  # EdgeInfos records kf->LEFT for every edge (src/BAoptimizer.cpp:107)

    def getEdgeSize(self) -> int:
        return self.s.n_edges

    def _sync_flags(self):
        if self._dirty_levels:
            self.s.set_levels(self._levels)
            self._dirty_levels = False
        if self._dirty_robust:
            self.s.set_robust(self._robust)
            self._dirty_robust = False

    # src/BAoptimizer.cpp:110-114
    def optimize(self, n: int) -> dict:
        self._sync_flags()
        st = self.s.optimize(n)
        self._chi2 = np.zeros(0)
        return st

    def _refresh_chi2(self):
        if len(self._chi2) != self.s.n_edges:
            self._sync_flags()
            self._chi2 = self.s.edge_chi2()

    def DumpCalculationGraph(self, file_name: str) -> None:
        self.s.dump_hessian(file_name)

    # src/BAoptimizer.cpp:121-132
    def eval(self, v):
        if isinstance(v, KeyFrame):
            return self.s.keyframe(self.KF2ID[id(v)])
        return self.s.mappoint(self.MP2ID[id(v)])

    # include/BAoptimizer.hpp:70-73
    def filter(self, callback: Callable) -> None:
        self._chi2 = np.zeros(0)
        for e, info in list(self.EdgeInfos.items()):
            callback((e, info))
        self._sync_flags()

    # src/BAoptimizer.cpp:134-143
    def recovery_all(self) -> None:
        for kf in self.ALLKFS.values():
            kf.Tcw = self.eval(kf)
        for mp in self.ALLMPS.values():
            mp.pos = self.eval(mp)

    def close(self):
        self.s.close()
