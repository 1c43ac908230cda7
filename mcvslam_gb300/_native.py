"""ctypes binding of libmcba.so (the C ABI in include/mcba.h).

The library is the only compute path: if it is missing or cannot be loaded
this module raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libmcba.so")

c_float_p = ctypes.POINTER(ctypes.c_float)
c_double_p = ctypes.POINTER(ctypes.c_double)
c_u8_p = ctypes.POINTER(ctypes.c_uint8)
c_i32_p = ctypes.POINTER(ctypes.c_int32)

MCBA_OK = 0
MCBA_ERR_TOO_LARGE = 9
NOALLOC_MAX_EDGES = 4096 * 256
STATUS = {0: "ok", 1: "invalid argument", 2: "nothing to optimise", 3: "not positive definite",
          4: "non-finite input", 5: "timeout", 6: "CUDA error", 7: "out of memory", 8: "no CUDA device",
          9: "too large"}


class Options(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int32), ("device", ctypes.c_int32), ("tau", ctypes.c_double),
                ("max_trials", ctypes.c_int32), ("use_graph", ctypes.c_int32), ("profile", ctypes.c_int32),
                ("stream", ctypes.c_void_p), ("host_structure", ctypes.c_int32)]


class Stats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int32), ("trials", ctypes.c_int32), ("n_active_edges", ctypes.c_int32),
                ("n_free_poses", ctypes.c_int32), ("n_free_points", ctypes.c_int32), ("status", ctypes.c_int32),
                ("initial_chi2", ctypes.c_double), ("final_chi2", ctypes.c_double), ("lambda_", ctypes.c_double),
                ("edges_linearized", ctypes.c_int64), ("ms_total", ctypes.c_double),
                ("ms_linearize", ctypes.c_double), ("ms_host_prepare", ctypes.c_double),
                ("ms_phase", ctypes.c_double * 8), ("n_phase", ctypes.c_int32 * 8),
                ("kernel_launches", ctypes.c_int64), ("h2d_bytes", ctypes.c_int64), ("d2h_bytes", ctypes.c_int64)]

    def as_dict(self) -> dict:
        d = {f: getattr(self, f) for f, _ in self._fields_}
        d["lambda"] = d.pop("lambda_")
        d["ms_phase"] = list(d["ms_phase"])
        d["n_phase"] = list(d["n_phase"])
        return d


PHASES = ["linearize", "reduce", "schur_edge", "schur_pairs", "schur_assemble", "cholesky", "update", "cost"]


class TrialLog(ctypes.Structure):
    _fields_ = [("iteration", ctypes.c_int32), ("trial", ctypes.c_int32), ("chi_before", ctypes.c_double),
                ("chi_after", ctypes.c_double), ("lambda_", ctypes.c_double), ("scale", ctypes.c_double),
                ("rho", ctypes.c_double), ("accepted", ctypes.c_int32), ("solve_ok", ctypes.c_int32)]


class ProblemDesc(ctypes.Structure):
    """mcba_problem_desc; pointer fields as plain host addresses (an address
    is assigned a quarter as fast as a typed ctypes pointer is built)."""
    _fields_ = [
        ("n_cams", ctypes.c_int32), ("cam_K", ctypes.c_void_p), ("cam_bf", ctypes.c_void_p),
        ("cam_Tcb", ctypes.c_void_p),
        ("n_poses", ctypes.c_int32), ("pose_Tcw", ctypes.c_void_p), ("pose_fixed", ctypes.c_void_p),
        ("n_points", ctypes.c_int32), ("point_Xw", ctypes.c_void_p), ("point_fixed", ctypes.c_void_p),
        ("n_edges", ctypes.c_int32), ("edge_type", ctypes.c_void_p), ("edge_pose", ctypes.c_void_p),
        ("edge_point", ctypes.c_void_p), ("edge_cam", ctypes.c_void_p), ("edge_obs", ctypes.c_void_p),
        ("edge_info", ctypes.c_void_p), ("edge_delta", ctypes.c_void_p), ("edge_robust", ctypes.c_void_p),
        ("edge_level", ctypes.c_void_p),
    ]


class ProjectionBatchDesc(ctypes.Structure):
    """mcba_projection_batch; pointer fields as plain addresses (host or device)."""
    _fields_ = [
        ("n_objects", ctypes.c_int32), ("obj_Rt", ctypes.c_void_p), ("obj_K", ctypes.c_void_p),
        ("obj_size", ctypes.c_void_p), ("obj_radius", ctypes.c_void_p), ("obj_scale", ctypes.c_void_p),
        ("n_levels", ctypes.c_int32), ("ratio", ctypes.c_float), ("max_dist", ctypes.c_int32),
        ("kp_begin", ctypes.c_void_p), ("kp_xy", ctypes.c_void_p), ("kp_desc", ctypes.c_void_p),
        ("mp_begin", ctypes.c_void_p), ("mp_X", ctypes.c_void_p), ("mp_desc", ctypes.c_void_p),
        ("mp_level", ctypes.c_void_p), ("mp_id", ctypes.c_void_p), ("mp_prev_kp", ctypes.c_void_p),
    ]


MAX_LEVELS = 32


class StereoBatchDesc(ctypes.Structure):
    """mcba_stereo_batch; pointer fields as plain addresses (host or device)."""
    _fields_ = [
        ("n_frames", ctypes.c_int32), ("n_levels", ctypes.c_int32),
        ("scale", ctypes.c_float * MAX_LEVELS), ("inv_scale", ctypes.c_float * MAX_LEVELS),
        ("level_rows", ctypes.c_int32 * MAX_LEVELS), ("level_cols", ctypes.c_int32 * MAX_LEVELS),
        ("level_offset", ctypes.c_int64 * MAX_LEVELS), ("pyr_bytes", ctypes.c_int64),
        ("image_rows", ctypes.c_int32), ("b", ctypes.c_float), ("bf", ctypes.c_float),
        ("left_pyr", ctypes.c_void_p), ("right_pyr", ctypes.c_void_p),
        ("left_begin", ctypes.c_void_p), ("left_xy", ctypes.c_void_p), ("left_oct", ctypes.c_void_p),
        ("left_desc", ctypes.c_void_p), ("right_begin", ctypes.c_void_p), ("right_xy", ctypes.c_void_p),
        ("right_oct", ctypes.c_void_p), ("right_desc", ctypes.c_void_p),
    ]


class MapDesc(ctypes.Structure):
    """mcba_map_desc (host arrays)."""
    _fields_ = [
        ("n_keyframes", ctypes.c_int32), ("kf_id", ctypes.c_void_p), ("kf_Tcw", ctypes.c_void_p),
        ("obs_begin", ctypes.c_void_p), ("obs_point", ctypes.c_void_p), ("obs_object", ctypes.c_void_p),
        ("obs_uv", ctypes.c_void_p), ("obs_ur", ctypes.c_void_p), ("obs_octave", ctypes.c_void_p),
        ("n_points", ctypes.c_int32), ("mp_Xw", ctypes.c_void_p), ("mp_kf_begin", ctypes.c_void_p),
        ("mp_kf", ctypes.c_void_p), ("ess_begin", ctypes.c_void_p), ("ess_adj", ctypes.c_void_p),
        ("n_levels", ctypes.c_int32), ("inv_sigma2_left", ctypes.c_void_p), ("inv_sigma2_wide", ctypes.c_void_p),
        ("K_left", ctypes.c_float * 4), ("K_wide", ctypes.c_float * 4), ("T_wide_body", ctypes.c_float * 16),
        ("bf", ctypes.c_float),
    ]


class WindowInfo(ctypes.Structure):
    _fields_ = [("n_local", ctypes.c_int32), ("n_anchor", ctypes.c_int32), ("n_poses", ctypes.c_int32),
                ("n_points", ctypes.c_int32), ("n_fixed_points", ctypes.c_int32), ("n_edges", ctypes.c_int32)]


_LIB = None


def _declare(L):
    P = ctypes.c_void_p
    i32 = ctypes.c_int32
    sig = {
        "mcba_abi_version": ([], ctypes.c_int),
        "mcba_status_string": ([ctypes.c_int], ctypes.c_char_p),
        "mcba_default_options": ([ctypes.POINTER(Options)], None),
        "mcba_device_count": ([ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
        "mcba_release_cached": ([i32], ctypes.c_int),
        "mcba_create": ([ctypes.POINTER(Options), ctypes.POINTER(P)], ctypes.c_int),
        "mcba_destroy": ([P], ctypes.c_int),
        "mcba_last_error": ([P], ctypes.c_char_p),
        "mcba_clear": ([P], ctypes.c_int),
        "mcba_add_camera": ([P, c_float_p, ctypes.c_float, c_float_p, c_i32_p], ctypes.c_int),
        "mcba_add_keyframe": ([P, c_float_p, ctypes.c_int, c_i32_p], ctypes.c_int),
        "mcba_add_keyframe_qt": ([P, c_double_p, ctypes.c_int, c_i32_p], ctypes.c_int),
        "mcba_add_mappoint": ([P, c_float_p, ctypes.c_int, c_i32_p], ctypes.c_int),
        "mcba_add_edge_mono": ([P, i32, i32, i32, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                c_i32_p], ctypes.c_int),
        "mcba_add_edge_stereo": ([P, i32, i32, i32, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                  ctypes.c_float, c_i32_p], ctypes.c_int),
        "mcba_add_edge_posonly": ([P, i32, i32, c_float_p, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                   ctypes.c_float, c_i32_p], ctypes.c_int),
        "mcba_add_edges": ([P, i32, c_u8_p, c_i32_p, c_i32_p, c_i32_p, c_float_p, c_float_p, c_float_p, c_float_p,
                            c_i32_p], ctypes.c_int),
        "mcba_load": ([P, ctypes.POINTER(ProblemDesc)], ctypes.c_int),
        "mcba_edge_count": ([P, c_i32_p], ctypes.c_int),
        "mcba_vertex_count": ([P, c_i32_p, c_i32_p], ctypes.c_int),
        "mcba_optimize": ([P, i32, ctypes.POINTER(Stats)], ctypes.c_int),
        "mcba_prepare": ([P], ctypes.c_int),
        "mcba_solve_prepared": ([P, i32, ctypes.POINTER(Stats)], ctypes.c_int),
        "mcba_batch_prepare": ([ctypes.POINTER(P), i32], ctypes.c_int),
        "mcba_batch_solve": ([ctypes.POINTER(P), i32, i32, ctypes.POINTER(Stats), c_double_p], ctypes.c_int),
        "mcba_batch_solve_persistent": ([ctypes.POINTER(P), i32, i32, ctypes.POINTER(Stats), c_double_p,
                                         ctypes.POINTER(i32)], ctypes.c_int),
        "mcba_fetch_state": ([P], ctypes.c_int),
        "mcba_trial_log_get": ([P, ctypes.POINTER(TrialLog), i32, c_i32_p], ctypes.c_int),
        "mcba_edge_chi2": ([P, c_double_p], ctypes.c_int),
        "mcba_set_edge_levels": ([P, c_u8_p], ctypes.c_int),
        "mcba_get_edge_levels": ([P, c_u8_p], ctypes.c_int),
        "mcba_set_edge_robust": ([P, c_u8_p], ctypes.c_int),
        "mcba_get_keyframe": ([P, i32, c_float_p], ctypes.c_int),
        "mcba_get_keyframe_qt": ([P, i32, c_double_p], ctypes.c_int),
        "mcba_get_mappoint": ([P, i32, c_float_p], ctypes.c_int),
        "mcba_get_state": ([P, c_double_p, c_double_p], ctypes.c_int),
        "mcba_set_state": ([P, c_double_p, c_double_p], ctypes.c_int),
        "mcba_dump_hessian": ([P, ctypes.c_char_p], ctypes.c_int),
        "mcba_pose_optimization": ([P, i32, i32, ctypes.c_float, i32, c_i32_p, c_i32_p], ctypes.c_int),
        "mcba_local_ba": ([P, i32, ctypes.c_float, c_i32_p, c_i32_p], ctypes.c_int),
        "mcba_local_window": ([P, ctypes.POINTER(MapDesc), i32, i32, c_u8_p, c_i32_p, c_i32_p, c_u8_p,
                               ctypes.POINTER(WindowInfo)], ctypes.c_int),
        "mcba_reproj_forward": ([i32, ctypes.c_int64, P, P, P, P, P, P, P, P, P], ctypes.c_int),
        "mcba_reproj_backward": ([i32, ctypes.c_int64, P, P, P, P, P, P, P, P, P, P, P, P, P, P], ctypes.c_int),
        "mcba_batch_pose_only": ([i32, i32, i32, c_i32_p, i32, c_float_p, c_float_p, c_i32_p, c_float_p, c_float_p,
                                  c_float_p, c_float_p, i32, i32, ctypes.c_float, i32, c_double_p, c_u8_p, c_i32_p,
                                  c_double_p], ctypes.c_int),
        "mcba_knn_hamming_device": ([P, i32, P, i32, P, P, ctypes.c_float, i32, P, P], ctypes.c_int),
        "mcba_knn_hamming": ([i32, c_u8_p, i32, c_u8_p, i32, c_i32_p, c_i32_p, ctypes.c_float, i32, c_u8_p,
                              c_double_p], ctypes.c_int),
        "mcba_project_match": ([i32, ctypes.POINTER(ProjectionBatchDesc), P, P, P, c_double_p], ctypes.c_int),
        "mcba_project_match_device": ([ctypes.POINTER(ProjectionBatchDesc), i32, i32, P, P, P, P], ctypes.c_int),
        "mcba_stereo_match": ([i32, ctypes.POINTER(StereoBatchDesc), P, P, c_double_p], ctypes.c_int),
        "mcba_stereo_match_device": ([ctypes.POINTER(StereoBatchDesc), i32, i32, P, P, P], ctypes.c_int),
        "mcba_fp64_fma_rate": ([i32, c_double_p], ctypes.c_int),
        "mcba_robust_cost_noalloc": ([ctypes.c_int64, P, P, P, P, P, P, P, P, P, P], ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    return L


def lib(build_if_missing: bool = True):
    """Load libmcba.so (building it first when it is missing or stale)."""
    global _LIB
    if _LIB is None:
        if build_if_missing:
            from mcvslam_gb300 import build as _build
            _build.build()
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libmcba.so not found at {LIB_PATH}; build it with mcvslam_gb300.build.build()")
        _LIB = _declare(ctypes.CDLL(LIB_PATH))
    return _LIB


class MCBAError(RuntimeError):
    def __init__(self, status: int, msg: str = ""):
        super().__init__(f"mcba status {status} ({STATUS.get(status, '?')}){': ' + msg if msg else ''}")
        self.status = status


def check(status: int, handle=None) -> int:
    if status != MCBA_OK:
        msg = ""
        if handle:
            m = lib().mcba_last_error(handle)
            msg = m.decode() if m else ""
        raise MCBAError(status, msg)
    return status


def device_count() -> int:
    n = ctypes.c_int(0)
    lib().mcba_device_count(ctypes.byref(n))
    return n.value
