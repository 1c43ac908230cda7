"""Brute-force Hamming k = 2 matching (Matcher::KnnMatch, src/Matcher.cpp:245-302)
on the GPU through libmcba.so.

Descriptors are 32-byte ORB descriptors ([n, 32] uint8).  Results follow the
reference's loop exactly: the best and second-best train index and distance
per query (ties to the smaller index, (999, 0) when fewer than two train
descriptors exist), plus the keep flag of FilterRatio / FilterThreshold.
"""
from __future__ import annotations

import ctypes

import numpy as np

from mcvslam_gb300 import _native as N


def knn_hamming(query, train, ratio: float = 0.6, max_dist: int = 46, device: int = 0):
    """Host arrays in, host arrays out: (idx [nq, 2], dist [nq, 2], keep [nq], kernel ms)."""
    q = np.ascontiguousarray(query, np.uint8).reshape(-1, 32)
    t = np.ascontiguousarray(train, np.uint8).reshape(-1, 32)
    nq, nt = q.shape[0], t.shape[0]
    idx = np.zeros((nq, 2), np.int32)
    dist = np.zeros((nq, 2), np.int32)
    keep = np.zeros(nq, np.uint8)
    ms = ctypes.c_double(0.0)
    N.check(N.lib().mcba_knn_hamming(device, q.ctypes.data_as(N.c_u8_p), nq, t.ctypes.data_as(N.c_u8_p), nt,
                                     idx.ctypes.data_as(N.c_i32_p), dist.ctypes.data_as(N.c_i32_p), ratio, max_dist,
                                     keep.ctypes.data_as(N.c_u8_p), ctypes.byref(ms)))
    return idx, dist, keep, ms.value


def knn_hamming_device(query, train, ratio: float = 0.6, max_dist: int = 46):
    """torch uint8 CUDA tensors [n, 32] in, CUDA tensors out (no host copies)."""
    import torch

    if not (query.is_cuda and train.is_cuda) or query.dtype != torch.uint8 or train.dtype != torch.uint8:
        raise ValueError("query and train must be uint8 CUDA tensors")
    q = query.contiguous().view(-1, 32)
    t = train.contiguous().view(-1, 32)
    nq, nt = q.shape[0], t.shape[0]
    idx = torch.empty((nq, 2), dtype=torch.int32, device=q.device)
    dist = torch.empty((nq, 2), dtype=torch.int32, device=q.device)
    keep = torch.empty(nq, dtype=torch.uint8, device=q.device)
    stream = torch.cuda.current_stream(q.device).cuda_stream
    N.check(N.lib().mcba_knn_hamming_device(q.data_ptr(), nq, t.data_ptr(), nt, idx.data_ptr(), dist.data_ptr(),
                                            ratio, max_dist, keep.data_ptr(), stream))
    return idx, dist, keep


_PB_FIELDS = [("obj_Rt", "float32"), ("obj_K", "float32"), ("obj_size", "int32"), ("obj_radius", "float32"),
              ("obj_scale", "float32"), ("kp_begin", "int32"), ("kp_xy", "float32"), ("kp_desc", "uint8"),
              ("mp_begin", "int32"), ("mp_X", "float32"), ("mp_desc", "uint8"), ("mp_level", "int32"),
              ("mp_id", "int32"), ("mp_prev_kp", "int32")]


def _batch_desc(b, arrays):
    d = N.ProjectionBatchDesc()
    d.n_objects = b.n_objects
    d.n_levels = int(b.obj_scale.shape[1])
    d.ratio = float(b.ratio)
    d.max_dist = int(b.max_dist)
    for name, _ in _PB_FIELDS:
        a = arrays.get(name)
        setattr(d, name, None if a is None else (a.data_ptr() if hasattr(a, "data_ptr") else a.ctypes.data))
    return d


def project_match(b, device: int = 0):
    """Object::ProjectBunchMapPoints over a batch of objects (host arrays of a
    synth.ProjectionBatch-like object): (kp_bind after the call, mp_match,
    obj_count, kernel ms)."""
    arrays = {}
    for name, dt in _PB_FIELDS:
        v = getattr(b, name, None)
        arrays[name] = None if v is None else np.ascontiguousarray(v, dtype=dt)
    d = _batch_desc(b, arrays)
    nk, nm = int(b.kp_begin[-1]), int(b.mp_begin[-1])
    kp_bind = np.array(b.kp_bind, np.int32, copy=True)
    mp_match = np.zeros(nm, np.int32)
    count = np.zeros(b.n_objects, np.int32)
    ms = ctypes.c_double(0.0)
    N.check(N.lib().mcba_project_match(device, ctypes.byref(d), kp_bind.ctypes.data, mp_match.ctypes.data,
                                       count.ctypes.data, ctypes.byref(ms)))
    return kp_bind, mp_match, count, ms.value


class DeviceProjectionBatch:
    """A projection batch resident on the GPU (torch tensors), for repeated
    device-side calls without host copies."""

    def __init__(self, b, device: int = 0):
        import torch

        self.b = b
        self.dev = torch.device("cuda", device)
        self.t = {}
        for name, dt in _PB_FIELDS:
            v = getattr(b, name, None)
            if v is not None:
                self.t[name] = torch.from_numpy(np.ascontiguousarray(v, dtype=dt)).to(self.dev)
        self.kp_bind0 = torch.from_numpy(np.ascontiguousarray(b.kp_bind, np.int32)).to(self.dev)
        self.kp_bind = self.kp_bind0.clone()
        self.nk, self.nm = int(b.kp_begin[-1]), int(b.mp_begin[-1])
        self.mp_match = torch.empty(max(self.nm, 1), dtype=torch.int32, device=self.dev)
        self.count = torch.empty(max(b.n_objects, 1), dtype=torch.int32, device=self.dev)
        self.desc = _batch_desc(b, self.t)

    def reset(self):
        """Restore the bindings the batch started with (the call updates them in place)."""
        self.kp_bind.copy_(self.kp_bind0)

    def run(self, reset: bool = True):
        """One call on torch's current stream; reset restores the initial bindings first."""
        import torch

        if reset:
            self.reset()
        stream = torch.cuda.current_stream(self.dev).cuda_stream
        N.check(N.lib().mcba_project_match_device(ctypes.byref(self.desc), self.nk, self.nm, self.kp_bind.data_ptr(),
                                                  self.mp_match.data_ptr(), self.count.data_ptr(), stream))
        return self.kp_bind, self.mp_match[:self.nm], self.count[:self.b.n_objects]


_SB_FIELDS = [("left_pyr", "uint8"), ("right_pyr", "uint8"), ("left_begin", "int32"), ("left_xy", "float32"),
              ("left_oct", "int32"), ("left_desc", "uint8"), ("right_begin", "int32"), ("right_xy", "float32"),
              ("right_oct", "int32"), ("right_desc", "uint8")]


def _stereo_desc(sb, arrays):
    d = N.StereoBatchDesc()
    d.n_frames = sb.n_frames
    nl = int(sb.scale.shape[0])
    if nl > N.MAX_LEVELS:
        raise ValueError(f"at most {N.MAX_LEVELS} pyramid levels")
    d.n_levels = nl
    for i in range(nl):
        d.scale[i] = float(sb.scale[i])
        d.inv_scale[i] = float(sb.inv_scale[i])
        d.level_rows[i] = int(sb.level_rows[i])
        d.level_cols[i] = int(sb.level_cols[i])
        d.level_offset[i] = int(sb.level_offset[i])
    d.pyr_bytes = int(sb.pyr_bytes)
    d.image_rows = int(sb.image_rows)
    d.b = float(sb.b)
    d.bf = float(sb.bf)
    for name, _ in _SB_FIELDS:
        a = arrays[name]
        setattr(d, name, a.data_ptr() if hasattr(a, "data_ptr") else a.ctypes.data)
    return d


def stereo_match(sb, device: int = 0):
    """Frame::ComputeStereoMatch over a batch of frames (host arrays of a
    synth.StereoBatch-like object): (u_right, depth, kernel ms)."""
    arrays = {name: np.ascontiguousarray(getattr(sb, name), dtype=dt) for name, dt in _SB_FIELDS}
    d = _stereo_desc(sb, arrays)
    nl = int(sb.left_begin[-1])
    u = np.zeros(nl, np.float32)
    z = np.zeros(nl, np.float32)
    ms = ctypes.c_double(0.0)
    N.check(N.lib().mcba_stereo_match(device, ctypes.byref(d), u.ctypes.data, z.ctypes.data, ctypes.byref(ms)))
    return u, z, ms.value


class DeviceStereoBatch:
    """A stereo batch resident on the GPU, for repeated device-side calls."""

    def __init__(self, sb, device: int = 0):
        import torch

        self.dev = torch.device("cuda", device)
        self.t = {name: torch.from_numpy(np.ascontiguousarray(getattr(sb, name), dtype=dt)).to(self.dev)
                  for name, dt in _SB_FIELDS}
        self.nl, self.nr = int(sb.left_begin[-1]), int(sb.right_begin[-1])
        self.u = torch.empty(max(self.nl, 1), dtype=torch.float32, device=self.dev)
        self.z = torch.empty(max(self.nl, 1), dtype=torch.float32, device=self.dev)
        self.desc = _stereo_desc(sb, self.t)

    def run(self):
        import torch

        stream = torch.cuda.current_stream(self.dev).cuda_stream
        N.check(N.lib().mcba_stereo_match_device(ctypes.byref(self.desc), self.nl, self.nr, self.u.data_ptr(),
                                                 self.z.data_ptr(), stream))
        return self.u[:self.nl], self.z[:self.nl]
