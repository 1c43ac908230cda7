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
