"""Seeded synthetic bundle-adjustment problems for the multi-camera rig.

The reference measures its local BA on an OpenSceneGraph-rendered drone
sequence that is not available; these generators stand in for it with the
shapes, sizes and noise model of the benchmark configurations:

* rig: left/right 640x480 cameras yawed 30 deg outward at x = 0 and x = 1.0 m,
  a 1280x720 wide camera (110 deg HFOV) at x = 0.5 m, all on one body;
* a smooth random drone trajectory (0.3 m steps, at most 5 deg per step);
* map points uniform in a 20 x 20 x 10 m box;
* every in-image projection with depth > 0.5 m kept, 2..8 per point;
* pixel noise N(0, 1 px^2), a fraction replaced by uniform outliers;
* initial poses perturbed N(0, 0.05 m / 1 deg), points N(0, 0.1 m);
* the first two keyframes fixed (and left unperturbed).

Everything crosses the boundary the way the reference hands it to
``BAoptimizer``: poses as float 4x4 T_body_world (``Frame::GetPose``), points
as float[3], observations as float pixels, information as float invSigma2,
Huber thresholds as float (include/BAoptimizer.hpp:62-63).

Body/camera frames follow the camera convention (x right, y down, z forward).
"""
from __future__ import annotations

import dataclasses
import math
from typing import Optional

import numpy as np

EDGE_MONO = 0
EDGE_STEREO = 1
EDGE_UNARY = 2

HUBER_BENCH = np.float32(math.sqrt(5.991))   # delta used by the benchmark configs
HUBER_2D = np.float32(math.sqrt(5.99))       # BAoptimizer::thHuber2D
HUBER_3D = np.float32(math.sqrt(7.815))      # BAoptimizer::thHuber3D


@dataclasses.dataclass
class Problem:
    """A bundle-adjustment problem in the layout of the C-ABI bulk loader."""

    cam_K: np.ndarray        # float32 [C, 4] fx fy cx cy
    cam_bf: np.ndarray       # float32 [C]
    cam_Tcb: np.ndarray      # float32 [C, 16] row-major T_cam_body
    cam_size: np.ndarray     # int32 [C, 2] width height (generator metadata)
    pose_Tcw: np.ndarray     # float32 [K, 16] row-major T_body_world
    pose_fixed: np.ndarray   # uint8 [K]
    point_Xw: np.ndarray     # float32 [P, 3]
    point_fixed: np.ndarray  # uint8 [P]
    edge_type: np.ndarray    # uint8 [E]
    edge_pose: np.ndarray    # int32 [E]
    edge_point: np.ndarray   # int32 [E]
    edge_cam: np.ndarray     # int32 [E]
    edge_obs: np.ndarray     # float32 [E, 3] u v u_right
    edge_info: np.ndarray    # float32 [E]
    edge_delta: np.ndarray   # float32 [E]
    edge_robust: np.ndarray  # uint8 [E]
    edge_level: np.ndarray   # uint8 [E]
    gt_pose_Tcw: Optional[np.ndarray] = None  # float64 [K, 4, 4]
    gt_point_Xw: Optional[np.ndarray] = None  # float64 [P, 3]
    name: str = ""

    @property
    def n_cams(self) -> int:
        return int(self.cam_K.shape[0])

    @property
    def n_poses(self) -> int:
        return int(self.pose_Tcw.shape[0])

    @property
    def n_points(self) -> int:
        return int(self.point_Xw.shape[0])

    @property
    def n_edges(self) -> int:
        return int(self.edge_type.shape[0])

    def copy(self) -> "Problem":
        return dataclasses.replace(self, **{f.name: (getattr(self, f.name).copy()
                                                      if isinstance(getattr(self, f.name), np.ndarray)
                                                      else getattr(self, f.name))
                                            for f in dataclasses.fields(self)})

    def arrays(self) -> dict:
        return {f.name: getattr(self, f.name) for f in dataclasses.fields(self)
                if isinstance(getattr(self, f.name), np.ndarray)}

    def save(self, path: str) -> None:
        np.savez_compressed(path, name=np.array(self.name), **self.arrays())

    @staticmethod
    def load(path: str) -> "Problem":
        z = np.load(path, allow_pickle=False)
        kw = {k: z[k] for k in z.files if k != "name"}
        for f in dataclasses.fields(Problem):
            if f.name not in kw and f.name != "name":
                kw[f.name] = None
        return Problem(name=str(z["name"]) if "name" in z.files else "", **kw)


# ----------------------------------------------------------------- geometry --
def rot_y(a: float) -> np.ndarray:
    c, s = math.cos(a), math.sin(a)
    return np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])


def so3_exp(w: np.ndarray) -> np.ndarray:
    """Rodrigues' formula for a batch of rotation vectors [..., 3]."""
    w = np.asarray(w, dtype=np.float64)
    th = np.linalg.norm(w, axis=-1)[..., None, None]
    K = np.zeros(w.shape[:-1] + (3, 3))
    K[..., 0, 1] = -w[..., 2]
    K[..., 0, 2] = w[..., 1]
    K[..., 1, 0] = w[..., 2]
    K[..., 1, 2] = -w[..., 0]
    K[..., 2, 0] = -w[..., 1]
    K[..., 2, 1] = w[..., 0]
    small = th < 1e-12
    ths = np.where(small, 1.0, th)
    a = np.where(small, 1.0, np.sin(ths) / ths)
    b = np.where(small, 0.5, (1 - np.cos(ths)) / (ths * ths))
    return np.eye(3) + a * K + b * (K @ K)


def make_T(R: np.ndarray, t: np.ndarray) -> np.ndarray:
    T = np.zeros(R.shape[:-2] + (4, 4))
    T[..., :3, :3] = R
    T[..., :3, 3] = t
    T[..., 3, 3] = 1.0
    return T


def inv_T(T: np.ndarray) -> np.ndarray:
    R = T[..., :3, :3]
    t = T[..., :3, 3]
    Rt = np.swapaxes(R, -1, -2)
    return make_T(Rt, -(Rt @ t[..., None])[..., 0])


def random_rotations(rng: np.random.Generator, n: int) -> np.ndarray:
    """Rotations uniform on SO(3) (normalised Gaussian quaternions)."""
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    x, y, z, w = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z)
    R[:, 0, 1] = 2 * (x * y - z * w)
    R[:, 0, 2] = 2 * (x * z + y * w)
    R[:, 1, 0] = 2 * (x * y + z * w)
    R[:, 1, 1] = 1 - 2 * (x * x + z * z)
    R[:, 1, 2] = 2 * (y * z - x * w)
    R[:, 2, 0] = 2 * (x * z - y * w)
    R[:, 2, 1] = 2 * (y * z + x * w)
    R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return R


# ---------------------------------------------------------------------- rig --
@dataclasses.dataclass
class Rig:
    K: np.ndarray       # [C, 4] float32
    size: np.ndarray    # [C, 2]
    T_cb: np.ndarray    # [C, 4, 4] float64 T_cam_body
    bf: np.ndarray      # [C] float32


def baseline_rig(narrow_hfov_deg: float = 30.0, yaw_deg: float = 30.0) -> Rig:
    """Left/right 640x480 at x=0 / x=1.0 m yawed outward, wide 1280x720 110 deg at x=0.5 m."""
    fn = 320.0 / math.tan(math.radians(narrow_hfov_deg) / 2)
    fw = 640.0 / math.tan(math.radians(110.0) / 2)
    K = np.array([[fn, fn, 320.0, 240.0], [fn, fn, 320.0, 240.0], [fw, fw, 640.0, 360.0]], dtype=np.float32)
    size = np.array([[640, 480], [640, 480], [1280, 720]], dtype=np.int32)
    y = math.radians(yaw_deg)
    T_bc = np.stack([make_T(rot_y(-y), np.array([0.0, 0, 0])),
                     make_T(rot_y(+y), np.array([1.0, 0, 0])),
                     make_T(np.eye(3), np.array([0.5, 0, 0]))])
    bf = np.array([fn * 1.0, fn * 1.0, 0.0], dtype=np.float32)
    return Rig(K=K, size=size, T_cb=inv_T(T_bc), bf=bf)


def reference_rig() -> Rig:
    """The reference's own rig: three 512x512 cameras (config/*.yaml), left = body."""
    K = np.array([[955.40503, 955.40503, 256.0, 256.0],
                  [955.40503, 955.40503, 256.0, 256.0],
                  [179.25313, 179.25313, 256.0, 256.0]], dtype=np.float32)
    size = np.array([[512, 512]] * 3, dtype=np.int32)
    T_bc = np.stack([np.eye(4), make_T(np.eye(3), np.array([1.0, 0, 0])),
                     make_T(np.eye(3), np.array([0.5, 0, 0]))])
    bf = np.array([955.40503, 955.40503, 0.0], dtype=np.float32)
    return Rig(K=K, size=size, T_cb=inv_T(T_bc), bf=bf)


# --------------------------------------------------------------- trajectory --
def drone_trajectory(rng: np.random.Generator, n: int, step: float = 0.3,
                     max_rot_deg: float = 5.0) -> np.ndarray:
    """World-from-body poses [n, 4, 4] of a smooth random drone path."""
    T_wb = np.zeros((n, 4, 4))
    R = np.eye(3)
    p = np.zeros(3)
    yaw_rate = 0.0
    heading = np.array([0.0, 0.0, 1.0])
    lim = math.radians(max_rot_deg)
    for k in range(n):
        T_wb[k] = make_T(R, p)
        yaw_rate = float(np.clip(yaw_rate + rng.normal(0, math.radians(1.0)), -math.radians(4.0), math.radians(4.0)))
        w = np.array([rng.normal(0, math.radians(0.5)), yaw_rate, rng.normal(0, math.radians(0.5))])
        ang = np.linalg.norm(w)
        if ang > lim:
            w *= lim / ang
        R = R @ so3_exp(w)
        drift = rng.normal(0, 0.15, 3)
        drift[1] *= 0.3
        heading = 0.8 * heading + 0.2 * (R[:, 2] + drift)
        heading /= np.linalg.norm(heading)
        p = p + step * heading
    return T_wb


# ------------------------------------------------------------------ helpers --
def _project(K: np.ndarray, Pc: np.ndarray) -> np.ndarray:
    z = Pc[..., 2]
    u = K[0] * Pc[..., 0] / z + K[2]
    v = K[1] * Pc[..., 1] / z + K[3]
    return np.stack([u, v], axis=-1)


def _perturb_pose(rng, T_bw: np.ndarray, rot_deg: float, trans_m: float) -> np.ndarray:
    T_wb = inv_T(T_bw)
    dR = so3_exp(rng.normal(0, math.radians(rot_deg), 3))
    T_wb2 = make_T(T_wb[:3, :3] @ dR, T_wb[:3, 3] + rng.normal(0, trans_m, 3))
    return inv_T(T_wb2)


def _finish(rig: Rig, T_bw_true, T_bw_init, pose_fixed, X_true, X_init, point_fixed,
            e_pose, e_point, e_cam, obs, e_type=None, delta=HUBER_BENCH, name="") -> Problem:
    E = len(e_pose)
    if e_type is None:
        e_type = np.zeros(E, np.uint8)
    obs3 = np.zeros((E, 3), np.float32)
    obs3[:, : obs.shape[1]] = obs
    return Problem(
        cam_K=rig.K.astype(np.float32), cam_bf=rig.bf.astype(np.float32),
        cam_Tcb=rig.T_cb.astype(np.float32).reshape(-1, 16), cam_size=rig.size.astype(np.int32),
        pose_Tcw=T_bw_init.astype(np.float32).reshape(-1, 16), pose_fixed=pose_fixed.astype(np.uint8),
        point_Xw=X_init.astype(np.float32), point_fixed=point_fixed.astype(np.uint8),
        edge_type=np.asarray(e_type, np.uint8), edge_pose=np.asarray(e_pose, np.int32),
        edge_point=np.asarray(e_point, np.int32), edge_cam=np.asarray(e_cam, np.int32),
        edge_obs=obs3, edge_info=np.ones(E, np.float32),
        edge_delta=np.full(E, delta, np.float32), edge_robust=np.ones(E, np.uint8),
        edge_level=np.zeros(E, np.uint8), gt_pose_Tcw=T_bw_true, gt_point_Xw=X_true, name=name)


# ----------------------------------------------------------------- local BA --
def local_ba(n_kf: int, n_points: int, seed: int, outlier_frac: float = 0.05,
             n_fixed: int = 2, rig: Optional[Rig] = None, box_offset: float = 0.0,
             max_obs: int = 8, corridor: bool = False, name: str = "") -> Problem:
    """Local-BA window: n_kf keyframes x 3 cameras observing n_points map points."""
    rng = np.random.default_rng(seed)
    rig = rig or baseline_rig()
    T_wb = drone_trajectory(rng, n_kf)
    T_bw = inv_T(T_wb)
    # box 20 (x) x 10 (y, vertical) x 20 (z) m, centred ahead of the mid trajectory
    if corridor:
        # large maps: each point lives in a 20 x 10 x 20 m box ahead of a
        # random keyframe, so the map follows the whole trajectory
        anchor = rng.integers(0, n_kf, n_points)
        centre = T_wb[anchor, :3, 3] + T_wb[anchor, :3, 2] * (10.0 + box_offset)
        X = centre + rng.uniform(-0.5, 0.5, (n_points, 3)) * np.array([20.0, 10.0, 20.0])
    else:
        # box 20 (x) x 10 (y, vertical) x 20 (z) m, centred ahead of the mid trajectory
        mid = T_wb[n_kf // 2, :3, 3]
        fwd = T_wb[n_kf // 2, :3, 2]
        centre = mid + fwd * (10.0 + box_offset)
        X = centre + rng.uniform(-0.5, 0.5, (n_points, 3)) * np.array([20.0, 10.0, 20.0])
    # visibility of every point in every camera, one keyframe at a time
    C = rig.K.shape[0]
    T_cw = rig.T_cb[None, :, :, :] @ T_bw[:, None, :, :]          # [K, C, 4, 4]
    vk_l, vc_l, vp_l, uv_l = [], [], [], []
    for k in range(n_kf):
        for c in range(C):
            Pc = X @ T_cw[k, c, :3, :3].T + T_cw[k, c, :3, 3]
            ok = Pc[:, 2] > 0.5
            uv = _project(rig.K[c].astype(np.float64), Pc)
            w, h = rig.size[c]
            ok &= (uv[:, 0] >= 0) & (uv[:, 0] < w) & (uv[:, 1] >= 0) & (uv[:, 1] < h)
            idx = np.nonzero(ok)[0]
            vk_l.append(np.full(len(idx), k)); vc_l.append(np.full(len(idx), c))
            vp_l.append(idx); uv_l.append(uv[idx])
    vk = np.concatenate(vk_l); vc = np.concatenate(vc_l); vp = np.concatenate(vp_l)
    uvall = np.concatenate(uv_l)
    # per point: keep 2..max_obs observations (random subset when more)
    order = np.lexsort((rng.random(len(vp)), vp))
    vk, vc, vp, uvall = vk[order], vc[order], vp[order], uvall[order]
    counts = np.bincount(vp, minlength=n_points)
    starts = np.concatenate([[0], np.cumsum(counts)[:-1]])
    rank = np.arange(len(vp)) - starts[vp]
    keep = (rank < max_obs) & (counts[vp] >= 2)
    vk, vc, vp, uvall = vk[keep], vc[keep], vp[keep], uvall[keep]
    used = np.unique(vp)
    remap = -np.ones(n_points, np.int64)
    remap[used] = np.arange(len(used))
    X = X[used]
    vp = remap[vp]
    # edges in keyframe-major order (the way PoseEstimation walks keyframes)
    o = np.lexsort((vp, vc, vk))
    vk, vc, vp, z = vk[o], vc[o], vp[o], uvall[o]
    z = z + rng.normal(0, 1.0, z.shape)
    out = rng.random(len(vk)) < outlier_frac
    sz = rig.size[vc].astype(np.float64)
    z[out] = rng.uniform(0, 1, (int(out.sum()), 2)) * sz[out]
    # initial estimates
    fixed = np.zeros(n_kf, np.uint8)
    fixed[:n_fixed] = 1
    T_init = T_bw.copy()
    for k in range(n_fixed, n_kf):
        T_init[k] = _perturb_pose(rng, T_bw[k], 1.0, 0.05)
    X_init = X + rng.normal(0, 0.1, X.shape)
    return _finish(rig, T_bw, T_init, fixed, X, X_init, np.zeros(len(X), np.uint8),
                   vk, vp, vc, z, name=name or f"local_ba_{n_kf}kf_{n_points}pts")


def reference_style(seed: int, n_kf: int = 5, n_points: int = 300) -> Problem:
    """Small problem on the reference rig with all three edge kinds: stereo
    edges (left observations with a right-image match, Huber sqrt(7.815)),
    mono left edges (Huber sqrt(5.99)) and wide-camera edges to the body
    (Huber sqrt(7.815)), some fixed points -- the mix BoundleAdjustment builds
    (include/PoseEstimation.hpp:40-101)."""
    rng = np.random.default_rng(seed)
    rig = reference_rig()
    T_wb = drone_trajectory(rng, n_kf)
    T_bw = inv_T(T_wb)
    mid = T_wb[n_kf // 2, :3, 3]
    fwd = T_wb[n_kf // 2, :3, 2]
    X = mid + fwd * 12.0 + rng.uniform(-0.5, 0.5, (n_points, 3)) * np.array([16.0, 8.0, 12.0])
    ep, ex, ec, et, eo, ed = [], [], [], [], [], []
    for k in range(n_kf):
        for c in (0, 2):
            T = rig.T_cb[c] @ T_bw[k]
            Pc = X @ T[:3, :3].T + T[:3, 3]
            uv = _project(rig.K[c].astype(np.float64), Pc)
            w, h = rig.size[c]
            ok = (Pc[:, 2] > 0.5) & (uv[:, 0] >= 0) & (uv[:, 0] < w) & (uv[:, 1] >= 0) & (uv[:, 1] < h)
            for p in np.nonzero(ok)[0]:
                u = uv[p] + rng.normal(0, 1.0, 2)
                if c == 0:
                    ur = u[0] - float(rig.bf[0]) / Pc[p, 2] + rng.normal(0, 1.0)
                    stereo = rng.random() < 0.5 and (u[0] - ur) >= 1.0
                    ep.append(k); ex.append(p); ec.append(0)
                    et.append(EDGE_STEREO if stereo else EDGE_MONO)
                    eo.append([u[0], u[1], ur if stereo else 0.0])
                    ed.append(HUBER_3D if stereo else HUBER_2D)
                else:
                    ep.append(k); ex.append(p); ec.append(2); et.append(EDGE_MONO)
                    eo.append([u[0], u[1], 0.0]); ed.append(HUBER_3D)
    E = len(ep)
    eo = np.asarray(eo)
    out = rng.random(E) < 0.05
    eo[out, 0] = rng.uniform(0, 512, out.sum())
    eo[out, 1] = rng.uniform(0, 512, out.sum())
    seen = np.bincount(np.asarray(ex), minlength=n_points)
    fixed_pts = (rng.random(n_points) < 0.2).astype(np.uint8)
    fixed = np.zeros(n_kf, np.uint8)
    fixed[0] = 1
    T_init = T_bw.copy()
    for k in range(1, n_kf):
        T_init[k] = _perturb_pose(rng, T_bw[k], 0.5, 0.03)
    X_init = X + rng.normal(0, 0.05, X.shape) * (1 - fixed_pts[:, None])
    pr = _finish(rig, T_bw, T_init, fixed, X, X_init, fixed_pts, ep, ex, ec, eo.astype(np.float32),
                 e_type=et, name=f"reference_style_{seed}")
    pr.edge_delta = np.asarray(ed, np.float32)
    del seen
    return pr


# --------------------------------------------------------------- map tables --
@dataclasses.dataclass
class MapTables:
    """Flat tables of a SLAM map in the layout of mcba_map_desc: what
    Map::AddKeyFrame reads before its local BA (src/Map.cpp:140-145) --
    keyframes with their LEFT and WIDE observations, map points with the
    keyframes bound to them (MapPoint::GetAllKeyFrame), the essential graph."""
    kf_id: np.ndarray        # int64 [K] Frame::id
    kf_Tcw: np.ndarray       # float32 [K, 16] T_body_world
    obs_begin: np.ndarray    # int32 [K + 1]
    obs_point: np.ndarray    # int32 [O]
    obs_object: np.ndarray   # uint8 [O] 0 LEFT, 1 WIDE
    obs_uv: np.ndarray       # float32 [O, 2]
    obs_ur: np.ndarray       # float32 [O] u_right (-1: none)
    obs_octave: np.ndarray   # uint8 [O]
    mp_Xw: np.ndarray        # float32 [P, 3]
    mp_kf_begin: np.ndarray  # int32 [P + 1]
    mp_kf: np.ndarray        # int32 [B]
    ess_begin: np.ndarray    # int32 [K + 1]
    ess_adj: np.ndarray      # int32 [A]
    inv_sigma2_left: np.ndarray   # float32 [L]
    inv_sigma2_wide: np.ndarray   # float32 [L]
    K_left: np.ndarray       # float32 [4]
    K_wide: np.ndarray       # float32 [4]
    T_wide_body: np.ndarray  # float32 [16]
    bf: float = 0.0

    @property
    def n_keyframes(self) -> int:
        return int(self.kf_id.shape[0])

    @property
    def n_points(self) -> int:
        return int(self.mp_Xw.shape[0])


def map_tables(n_kf: int, n_points: int, seed: int, per_object: int = 300, stereo_frac: float = 0.5,
               unbound_frac: float = 0.02, n_levels: int = 8, ess_k: int = 4) -> MapTables:
    """A keyframe map on the reference rig (LEFT = body, WIDE camera, right
    image through u_right): n_kf keyframes on a drone path, n_points map points
    around it, at most per_object observations per keyframe and camera.  The
    last keyframe is the new one: like the reference at its local BA, its
    observations are not yet bound back to their map points (the binding
    follows the BA, src/Map.cpp:148-154); a few other bindings are missing at
    random.  Keyframe ids rise with gaps, the first is 0.  u_right values
    include some in [0, 1), which the BA treats as mono (MIN_DISPARITY = 1).
    Essential graph: each keyframe linked to its ess_k most covisible others."""
    rng = np.random.default_rng(seed)
    rig = reference_rig()
    T_wb = drone_trajectory(rng, n_kf)
    T_bw = inv_T(T_wb)
    anchor = rng.integers(0, n_kf, n_points)
    centre = T_wb[anchor, :3, 3] + T_wb[anchor, :3, 2] * 8.0
    X = centre + rng.uniform(-0.5, 0.5, (n_points, 3)) * np.array([16.0, 8.0, 10.0])
    cams = (0, 2)  # LEFT, WIDE of the rig
    ob_kf, ob_pt, ob_obj, ob_uv, ob_ur = [], [], [], [], []
    for k in range(n_kf):
        for o, c in enumerate(cams):
            Tcw = rig.T_cb[c] @ T_bw[k]
            Pc = X @ Tcw[:3, :3].T + Tcw[:3, 3]
            ok = Pc[:, 2] > 0.5
            uv = _project(rig.K[c].astype(np.float64), Pc)
            w, h = rig.size[c]
            ok &= (uv[:, 0] >= 0) & (uv[:, 0] < w) & (uv[:, 1] >= 0) & (uv[:, 1] < h)
            idx = np.nonzero(ok)[0]
            if len(idx) > per_object:
                idx = np.sort(rng.choice(idx, per_object, replace=False))
            idx = rng.permutation(idx)  # table order within an object is arbitrary
            z = uv[idx] + rng.normal(0, 1.0, (len(idx), 2))
            ur = np.full(len(idx), -1.0)
            if o == 0:
                st = rng.random(len(idx)) < stereo_frac
                ur[st] = z[st, 0] - rig.bf[0] / Pc[idx[st], 2]
                small = st & (rng.random(len(idx)) < 0.1)
                ur[small] = rng.uniform(0.0, 1.0, int(small.sum()))
            ob_kf.append(np.full(len(idx), k)); ob_pt.append(idx); ob_obj.append(np.full(len(idx), o))
            ob_uv.append(z); ob_ur.append(ur)
    kf = np.concatenate(ob_kf); pt = np.concatenate(ob_pt); obj = np.concatenate(ob_obj)
    uvs = np.concatenate(ob_uv); urs = np.concatenate(ob_ur)
    # interleave LEFT and WIDE rows inside a keyframe (the table need not be grouped)
    order = np.lexsort((rng.random(len(kf)), kf))
    kf, pt, obj, uvs, urs = kf[order], pt[order], obj[order], uvs[order], urs[order]
    obs_begin = np.zeros(n_kf + 1, np.int32)
    obs_begin[1:] = np.cumsum(np.bincount(kf, minlength=n_kf))
    # bindings point -> keyframe (set semantics), minus the new keyframe
    bound = (kf != n_kf - 1) & (rng.random(len(kf)) >= unbound_frac)
    pairs = np.unique(np.stack([pt[bound], kf[bound]], 1), axis=0) if bound.any() else np.zeros((0, 2), np.int64)
    # the binding list of a point in an arbitrary order
    pairs = pairs[np.lexsort((rng.random(len(pairs)), pairs[:, 0]))]
    mp_kf_begin = np.zeros(n_points + 1, np.int32)
    mp_kf_begin[1:] = np.cumsum(np.bincount(pairs[:, 0], minlength=n_points))
    # essential graph from covisibility
    M = np.zeros((n_kf, n_points), np.uint8)
    M[kf, pt] = 1
    cov = M.astype(np.int32) @ M.T.astype(np.int32)
    np.fill_diagonal(cov, 0)
    adj = [set() for _ in range(n_kf)]
    for k in range(n_kf):
        best = np.argsort(-cov[k], kind="stable")[:ess_k]
        for j in best:
            if cov[k, j] > 0:
                adj[k].add(int(j)); adj[int(j)].add(k)
    ess_begin = np.zeros(n_kf + 1, np.int32)
    ess_adj = []
    for k in range(n_kf):
        nb = rng.permutation(sorted(adj[k]))
        ess_adj.extend(int(x) for x in nb)
        ess_begin[k + 1] = len(ess_adj)
    ids = np.concatenate([[0], np.cumsum(rng.integers(1, 4, n_kf - 1))]).astype(np.int64)
    T_init = T_bw.copy()
    for k in range(2, n_kf):
        T_init[k] = _perturb_pose(rng, T_bw[k], 1.0, 0.05)
    X_init = X + rng.normal(0, 0.1, X.shape)
    scale = 1.2 ** np.arange(n_levels)
    inv_s2 = (1.0 / (scale * scale)).astype(np.float32)
    return MapTables(
        kf_id=ids, kf_Tcw=T_init.astype(np.float32).reshape(n_kf, 16), obs_begin=obs_begin,
        obs_point=pt.astype(np.int32), obs_object=obj.astype(np.uint8), obs_uv=uvs.astype(np.float32),
        obs_ur=urs.astype(np.float32), obs_octave=rng.integers(0, n_levels, len(kf)).astype(np.uint8),
        mp_Xw=X_init.astype(np.float32), mp_kf_begin=mp_kf_begin, mp_kf=pairs[:, 1].astype(np.int32),
        ess_begin=ess_begin, ess_adj=np.asarray(ess_adj, np.int32), inv_sigma2_left=inv_s2,
        inv_sigma2_wide=inv_s2.copy(), K_left=rig.K[0].copy(), K_wide=rig.K[2].copy(),
        T_wide_body=rig.T_cb[2].astype(np.float32).reshape(16), bf=float(rig.bf[0]))


# ---------------------------------------------------------------- pose-only --
def pose_only(n_obs: int, seed: int, outlier_frac: float = 0.10, rig: Optional[Rig] = None,
              delta=HUBER_BENCH) -> Problem:
    """One frame with n_obs observations of fixed map points (Tracker's
    pose-only optimisation, src/PoseEstimation.cpp:48-130): points sampled in
    the three cameras' frusta at depth U(1, 30) m, 10% outliers, the body
    pose perturbed N(0, 0.05 m / 1 deg)."""
    rng = np.random.default_rng(seed)
    rig = rig or baseline_rig()
    R = random_rotations(rng, 1)[0]
    T_wb = make_T(R, rng.normal(0, 5.0, 3))
    T_bw = inv_T(T_wb)
    cam = rng.integers(0, rig.K.shape[0], n_obs)
    sz = rig.size[cam].astype(np.float64)
    uv = rng.uniform(0, 1, (n_obs, 2)) * sz
    d = rng.uniform(1.0, 30.0, n_obs)
    K = rig.K[cam].astype(np.float64)
    Pc = np.stack([(uv[:, 0] - K[:, 2]) / K[:, 0] * d, (uv[:, 1] - K[:, 3]) / K[:, 1] * d, d], axis=1)
    T_wc = T_wb[None] @ inv_T(rig.T_cb)[cam]
    X = np.einsum("nij,nj->ni", T_wc[:, :3, :3], Pc) + T_wc[:, :3, 3]
    z = uv + rng.normal(0, 1.0, uv.shape)
    out = rng.random(n_obs) < outlier_frac
    z[out] = rng.uniform(0, 1, (int(out.sum()), 2)) * sz[out]
    T_init = _perturb_pose(rng, T_bw, 1.0, 0.05)
    return _finish(rig, T_bw[None], T_init[None], np.zeros(1, np.uint8), X, X,
                   np.ones(n_obs, np.uint8), np.zeros(n_obs, np.int64), np.arange(n_obs), cam, z,
                   delta=delta, name=f"pose_only_{n_obs}")


# ------------------------------------------------------------ random edges --
def random_edges(n: int, seed: int, rig: Optional[Rig] = None):
    """Independent mono edges for the differentiation check: body poses with
    rotations uniform on SO(3) and translations N(0, 5 m), the baseline rig's
    extrinsics, points at depth U(1, 50) m in front of their camera.

    Returns (T_bw [n,4,4] f64, T_cb [n,4,4] f64, K [n,4] f64, X [n,3] f64,
    obs [n,2] f64, cam [n] int)."""
    rng = np.random.default_rng(seed)
    rig = rig or baseline_rig()
    R = random_rotations(rng, n)
    T_wb = make_T(R, rng.normal(0, 5.0, (n, 3)))
    cam = rng.integers(0, rig.K.shape[0], n)
    K = rig.K[cam].astype(np.float64)
    sz = rig.size[cam].astype(np.float64)
    uv = rng.uniform(0, 1, (n, 2)) * sz
    d = rng.uniform(1.0, 50.0, n)
    Pc = np.stack([(uv[:, 0] - K[:, 2]) / K[:, 0] * d, (uv[:, 1] - K[:, 3]) / K[:, 1] * d, d], axis=1)
    T_wc = T_wb @ inv_T(rig.T_cb)[cam]
    X = np.einsum("nij,nj->ni", T_wc[:, :3, :3], Pc) + T_wc[:, :3, 3]
    obs = uv + rng.normal(0, 1.0, uv.shape)
    return inv_T(T_wb), rig.T_cb[cam], K, X, obs, cam


# ------------------------------------------------------------ named configs --
def window_batch(n: int = 64, seed: int = 4000, kf_range=(5, 40), pts_per_kf=(50, 300)) -> list:
    """Local-BA windows of the batched benchmark: n windows of U(5, 40)
    keyframes with U(50, 300) map points per keyframe (corridor layout, so
    points follow the trajectory), 5% outliers, first 2 keyframes fixed."""
    rng = np.random.default_rng(seed)
    out = []
    for w in range(n):
        k = int(rng.integers(kf_range[0], kf_range[1] + 1))
        ppk = int(rng.integers(pts_per_kf[0], pts_per_kf[1] + 1))
        out.append(local_ba(k, k * ppk, seed + 1 + w, corridor=True, name=f"window{w}_{k}kf"))
    return out


def config(idx: int, rep: int = 0) -> Problem:
    """Benchmark configurations (1-based, seed = idx * 1000 + rep).

    1: 10 keyframes, 2000 points (~9k edges); 2: 30 keyframes, 20k points
    (~150k observations); 5: 300 keyframes, 200k points (~2M observations)."""
    seed = idx * 1000 + rep
    if idx == 1:
        return local_ba(10, 2000, seed, box_offset=CONFIG_BOX_OFFSET[1], name="config1_10kf_2000pts")
    if idx == 2:
        return local_ba(30, 20000, seed, box_offset=CONFIG_BOX_OFFSET[2], name="config2_30kf_20kpts")
    if idx == 5:
        return local_ba(300, 200000, seed, box_offset=CONFIG_BOX_OFFSET[5], corridor=True,
                        name="config5_300kf_200kpts")
    raise ValueError(f"config {idx} is not a single local-BA problem")


# box placement that gives the configurations' edge counts (~9k / ~150k / ~2M)
CONFIG_BOX_OFFSET = {1: -4.0, 2: 0.0, 5: 0.0}


def descriptors(nq: int, nt: int, seed: int, match_frac: float = 0.6, flips: tuple = (0, 40)):
    """ORB-like 32-byte descriptor sets for the matcher: nt random train
    descriptors, and nq queries of which a fraction are copies of a random
    train descriptor with a uniform number of bits in [flips) flipped (a
    re-observation), the rest unrelated."""
    rng = np.random.default_rng(seed)
    train = rng.integers(0, 256, size=(nt, 32), dtype=np.uint8)
    query = rng.integers(0, 256, size=(nq, 32), dtype=np.uint8)
    if nt:
        m = rng.random(nq) < match_frac
        src = rng.integers(0, nt, size=nq)
        bits = np.unpackbits(train[src], axis=1)
        nflip = rng.integers(flips[0], flips[1], size=nq)
        for i in np.nonzero(m)[0]:
            b = bits[i].copy()
            pos = rng.choice(256, size=int(nflip[i]), replace=False)
            b[pos] ^= 1
            query[i] = np.packbits(b)
    return query, train


@dataclasses.dataclass
class ProjectionBatch:
    """Objects (one camera of one frame each) for Object::ProjectBunchMapPoints."""
    obj_Rt: np.ndarray      # [O, 12] float32: R row-major then t (camera from world)
    obj_K: np.ndarray       # [O, 4] float32
    obj_size: np.ndarray    # [O, 2] int32 cols, rows
    obj_radius: np.ndarray  # [O] float32
    obj_scale: np.ndarray   # [O, L] float32
    ratio: float
    max_dist: int
    kp_begin: np.ndarray    # [O+1] int32
    kp_xy: np.ndarray       # [NK, 2] float32
    kp_desc: np.ndarray     # [NK, 32] uint8
    kp_bind: np.ndarray     # [NK] int32 (map-point id or -1)
    mp_begin: np.ndarray    # [O+1] int32
    mp_X: np.ndarray        # [NM, 3] float32
    mp_desc: np.ndarray     # [NM, 32] uint8
    mp_level: np.ndarray    # [NM] int32
    mp_id: np.ndarray       # [NM] int32
    mp_prev_kp: np.ndarray  # [NM] int32 (object-local keypoint already bound to the map point, or -1)

    @property
    def n_objects(self):
        return int(self.obj_Rt.shape[0])


def scale_factors(n_levels: int = 8, factor: float = 1.2) -> np.ndarray:
    """ORB pyramid scale factors as ORBextractor fills mvScaleFactor (float,
    each level the previous times the double factor)."""
    s = np.zeros(n_levels, np.float32)
    s[0] = 1.0
    for i in range(1, n_levels):
        s[i] = np.float32(float(s[i - 1]) * factor)
    return s


def projection_batch(n_objects: int, n_kp: int, n_mp: int, seed: int, radius: float = 10.0,
                     rig: Optional[Rig] = None, observed_frac: float = 0.7, prebound_frac: float = 0.2,
                     dup_frac: float = 0.05) -> ProjectionBatch:
    """Each object: a camera looking down +z from a random pose near the origin,
    n_mp map points in front of it (a few behind it or outside the image),
    n_kp keypoints of which observed_frac of the map points leave one near
    their projection with a perturbed descriptor, the rest clutter.  Some
    keypoints start bound (to earlier map points, and to map points of this
    call, with mp_prev_kp consistent); dup_frac of the map points repeat
    another's descriptor and position, so several map points can claim one
    keypoint."""
    rng = np.random.default_rng(seed)
    rig = rig or reference_rig()
    O = n_objects
    cams = rng.integers(0, rig.K.shape[0], size=O)
    K = rig.K[cams].astype(np.float32)
    size = rig.size[cams].astype(np.int32)
    # small rotations only: cameras look roughly along +z
    w = rng.normal(0, 0.05, size=(O, 3))
    R = np.stack([so3_exp(wi) for wi in w])
    t = rng.normal(0, 0.2, size=(O, 3))
    Rt = np.concatenate([R.reshape(O, 9), t], axis=1).astype(np.float32)
    scale = np.tile(scale_factors(), (O, 1))
    kp_begin = np.arange(O + 1, dtype=np.int32) * n_kp
    mp_begin = np.arange(O + 1, dtype=np.int32) * n_mp
    kp_xy = np.zeros((O * n_kp, 2), np.float32)
    kp_desc = rng.integers(0, 256, size=(O * n_kp, 32), dtype=np.uint8)
    kp_bind = np.full(O * n_kp, -1, np.int32)
    mp_X = np.zeros((O * n_mp, 3), np.float32)
    mp_desc = rng.integers(0, 256, size=(O * n_mp, 32), dtype=np.uint8)
    mp_level = rng.integers(0, 8, size=O * n_mp).astype(np.int32)
    mp_id = (np.arange(O * n_mp, dtype=np.int64) * 7 + 1000).astype(np.int32)
    mp_prev = np.full(O * n_mp, -1, np.int32)
    next_free_id = int(mp_id.max()) + 1
    for o in range(O):
        cols, rows = int(size[o, 0]), int(size[o, 1])
        fx, fy, cx, cy = [float(v) for v in K[o]]
        # pixels and depths -> camera points -> world points
        u = rng.uniform(-0.05 * cols, 1.05 * cols, n_mp)
        v = rng.uniform(-0.05 * rows, 1.05 * rows, n_mp)
        z = rng.uniform(2.0, 30.0, n_mp)
        z[rng.random(n_mp) < 0.03] *= -1.0
        Pc = np.stack([(u - cx) / fx * z, (v - cy) / fy * z, z], axis=1)
        Xw = (Pc - t[o]) @ R[o]
        mX = mp_X[o * n_mp:(o + 1) * n_mp]
        mX[:] = Xw.astype(np.float32)
        md = mp_desc[o * n_mp:(o + 1) * n_mp]
        ml = mp_level[o * n_mp:(o + 1) * n_mp]
        ndup = int(dup_frac * n_mp)
        if ndup and n_mp > 1:
            src = rng.integers(0, n_mp, ndup)
            dst = rng.integers(0, n_mp, ndup)
            mX[dst] = mX[src]
            md[dst] = md[src]
            ml[dst] = ml[src]
        # keypoints: observations of map points, then clutter
        kx = kp_xy[o * n_kp:(o + 1) * n_kp]
        kd = kp_desc[o * n_kp:(o + 1) * n_kp]
        kx[:, 0] = rng.uniform(0, cols, n_kp)
        kx[:, 1] = rng.uniform(0, rows, n_kp)
        obs = np.nonzero(rng.random(n_mp) < observed_frac)[0][:n_kp]
        slots = rng.permutation(n_kp)[:obs.size]
        Xc = mX[obs].astype(np.float64) @ R[o].T + t[o]
        with np.errstate(divide="ignore", invalid="ignore"):
            pu = fx * Xc[:, 0] / Xc[:, 2] + cx
            pv = fy * Xc[:, 1] / Xc[:, 2] + cy
        ok = np.isfinite(pu) & np.isfinite(pv)
        kx[slots[ok], 0] = (pu[ok] + rng.normal(0, 1.5, ok.sum())).astype(np.float32)
        kx[slots[ok], 1] = (pv[ok] + rng.normal(0, 1.5, ok.sum())).astype(np.float32)
        bits = np.unpackbits(md[obs[ok]], axis=1)
        flips = rng.random(bits.shape) < rng.uniform(0.0, 0.15, size=(bits.shape[0], 1))
        kd[slots[ok]] = np.packbits(bits ^ flips.astype(np.uint8), axis=1)
        # pre-existing bindings: a few to foreign map points, a few to map points of this call
        kb = kp_bind[o * n_kp:(o + 1) * n_kp]
        mpv = mp_prev[o * n_mp:(o + 1) * n_mp]
        nb = int(prebound_frac * n_kp)
        free = rng.permutation(n_kp)[:nb]
        half = nb // 2
        for i in free[:half]:
            kb[i] = next_free_id
            next_free_id += 1
        own = rng.permutation(n_mp)[:nb - half]
        for i, m in zip(free[half:], own):
            kb[i] = mp_id[o * n_mp + m]
            mpv[m] = i
    return ProjectionBatch(obj_Rt=Rt, obj_K=K, obj_size=size, obj_radius=np.full(O, radius, np.float32),
                           obj_scale=scale.astype(np.float32), ratio=0.6, max_dist=46, kp_begin=kp_begin,
                           kp_xy=kp_xy, kp_desc=kp_desc, kp_bind=kp_bind, mp_begin=mp_begin, mp_X=mp_X,
                           mp_desc=mp_desc, mp_level=mp_level, mp_id=mp_id, mp_prev_kp=mp_prev)


@dataclasses.dataclass
class StereoBatch:
    """Rectified stereo frames for Frame::ComputeStereoMatch."""
    scale: np.ndarray        # [L] float32 mvScaleFactor
    inv_scale: np.ndarray    # [L] float32 mvInvScaleFactor
    level_rows: np.ndarray   # [L] int32
    level_cols: np.ndarray   # [L] int32
    level_offset: np.ndarray  # [L] int64 byte offset of each level in one image's pyramid
    pyr_bytes: int
    left_pyr: np.ndarray     # [F, pyr_bytes] uint8
    right_pyr: np.ndarray    # [F, pyr_bytes] uint8
    image_rows: int
    b: float
    bf: float
    left_begin: np.ndarray   # [F+1] int32
    left_xy: np.ndarray      # [NL, 2] float32
    left_oct: np.ndarray     # [NL] int32
    left_desc: np.ndarray    # [NL, 32] uint8
    right_begin: np.ndarray  # [F+1] int32
    right_xy: np.ndarray     # [NR, 2] float32
    right_oct: np.ndarray    # [NR] int32
    right_desc: np.ndarray   # [NR, 32] uint8

    @property
    def n_frames(self):
        return int(self.left_begin.shape[0] - 1)


def _texture(rng, rows, cols):
    """Smooth random uint8 texture (box-blurred noise at two scales)."""
    a = rng.random((rows + 8, cols + 8))
    # 5-tap box filter along each axis through cumulative sums
    c = np.cumsum(np.pad(a, ((0, 0), (3, 2))), axis=1)
    a = (c[:, 5:] - c[:, :-5]) / 5.0
    c = np.cumsum(np.pad(a, ((3, 2), (0, 0))), axis=0)
    a = (c[5:, :] - c[:-5, :]) / 5.0
    a = (a - a.min()) / max(np.ptp(a), 1e-9)
    return (a[4:4 + rows, 4:4 + cols] * 255).astype(np.uint8)


def stereo_batch(n_frames: int, n_left: int, n_right_clutter: int, seed: int, size=(512, 512),
                 fx: float = 955.40503, baseline: float = 1.0, n_levels: int = 8, match_frac: float = 0.8):
    """Each frame: a textured left pyramid, the right pyramid shifted by the
    frame's disparity (scaled per level) plus noise, n_left left keypoints
    (random octave, inside the ORB border), their right counterparts for
    match_frac of them (disparity + sub-pixel noise, perturbed descriptor,
    octave within one level) and n_right_clutter unrelated right keypoints."""
    rng = np.random.default_rng(seed)
    cols0, rows0 = size
    scale = scale_factors(n_levels)
    inv = (np.float32(1.0) / scale).astype(np.float32)
    lr = np.array([int(round(float(rows0) * float(s))) for s in inv], np.int32)
    lc = np.array([int(round(float(cols0) * float(s))) for s in inv], np.int32)
    off = np.zeros(n_levels, np.int64)
    for i in range(1, n_levels):
        off[i] = off[i - 1] + int(lr[i - 1]) * int(lc[i - 1])
    pyr_bytes = int(off[-1] + int(lr[-1]) * int(lc[-1]))
    left_pyr = np.zeros((n_frames, pyr_bytes), np.uint8)
    right_pyr = np.zeros((n_frames, pyr_bytes), np.uint8)
    L_xy, L_oct, L_desc, R_xy, R_oct, R_desc = [], [], [], [], [], []
    lb, rb = [0], [0]
    for f in range(n_frames):
        disp = float(rng.uniform(8.0, 60.0))
        for lev in range(n_levels):
            rows, cols = int(lr[lev]), int(lc[lev])
            shift = disp * float(inv[lev])
            s_int = int(np.floor(shift))
            tex = _texture(rng, rows, cols + s_int + 2)
            left = tex[:, s_int:s_int + cols]
            right = tex[:, :cols].astype(np.int16) + rng.integers(-3, 4, size=(rows, cols))
            left_pyr[f, off[lev]:off[lev] + rows * cols] = left.reshape(-1)
            right_pyr[f, off[lev]:off[lev] + rows * cols] = np.clip(right, 0, 255).astype(np.uint8).reshape(-1)
        oct_ = rng.integers(0, n_levels, n_left).astype(np.int32)
        margin = 19.0 * scale[oct_]
        x = rng.uniform(margin + disp + 12 * scale[oct_], cols0 - margin).astype(np.float32)
        y = rng.uniform(margin, rows0 - margin).astype(np.float32)
        desc = rng.integers(0, 256, size=(n_left, 32), dtype=np.uint8)
        L_xy.append(np.stack([x, y], 1))
        L_oct.append(oct_)
        L_desc.append(desc)
        m = rng.random(n_left) < match_frac
        xr = (x[m] - disp + rng.normal(0, 0.4, m.sum())).astype(np.float32)
        yr = (y[m] + rng.normal(0, 0.4, m.sum())).astype(np.float32)
        orr = np.clip(oct_[m] + rng.integers(-1, 2, m.sum()), 0, n_levels - 1).astype(np.int32)
        bits = np.unpackbits(desc[m], axis=1)
        flips = rng.random(bits.shape) < 0.04
        dr = np.packbits(bits ^ flips.astype(np.uint8), axis=1)
        oc = rng.integers(0, n_levels, n_right_clutter).astype(np.int32)
        mc = 19.0 * scale[oc]
        xc = rng.uniform(mc, cols0 - mc).astype(np.float32)
        yc = rng.uniform(mc, rows0 - mc).astype(np.float32)
        dc = rng.integers(0, 256, size=(n_right_clutter, 32), dtype=np.uint8)
        perm = rng.permutation(m.sum() + n_right_clutter)
        R_xy.append(np.concatenate([np.stack([xr, yr], 1), np.stack([xc, yc], 1)])[perm])
        R_oct.append(np.concatenate([orr, oc])[perm])
        R_desc.append(np.concatenate([dr, dc])[perm])
        lb.append(lb[-1] + n_left)
        rb.append(rb[-1] + int(m.sum()) + n_right_clutter)
    return StereoBatch(scale=scale, inv_scale=inv, level_rows=lr, level_cols=lc, level_offset=off,
                       pyr_bytes=pyr_bytes, left_pyr=left_pyr, right_pyr=right_pyr, image_rows=rows0,
                       b=float(baseline), bf=float(np.float32(fx * baseline)), left_begin=np.array(lb, np.int32),
                       left_xy=np.concatenate(L_xy).astype(np.float32), left_oct=np.concatenate(L_oct),
                       left_desc=np.concatenate(L_desc), right_begin=np.array(rb, np.int32),
                       right_xy=np.concatenate(R_xy).astype(np.float32), right_oct=np.concatenate(R_oct),
                       right_desc=np.concatenate(R_desc))
