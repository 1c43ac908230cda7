"""torch.autograd.Function over the reprojection residual kernels.

The residual of MCVSLAM's EdgeSE3XYZ2Camera (include/OptimizeTypes.hpp:80-86),

    r = obs - pi(T_cb * T_bw * X),

is computed by ``mcba_reproj_forward`` and its vector-Jacobian products by
``mcba_reproj_backward`` (libmcba.so).  Poses are parametrised the way g2o
perturbs them (VertexSE3Expmap::oplusImpl, types_six_dof_expmap.h:98-101):
the differentiable inputs are left perturbations delta (rotation first) of
the body pose and of the rig extrinsic, T <- exp(delta) T, plus the point X.
Gradients are taken on the tangent space at the perturbed pose; at delta = 0
they are exactly d r / d delta, which is what finite-difference checks and
optimisers built on g2o's convention use.

Only device tensors are accepted; float64 and float32 are supported.  This
module is a harness around the kernels -- there is no other implementation
behind it.
"""
from __future__ import annotations

import torch

from mcvslam_gb300 import _native as N


def _check(t: torch.Tensor, name: str, shape_tail, dtype) -> torch.Tensor:
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor")
    if t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype}, got {t.dtype}")
    if tuple(t.shape[1:]) != tuple(shape_tail):
        raise ValueError(f"{name} must have shape [n, {', '.join(map(str, shape_tail))}], got {tuple(t.shape)}")
    return t.contiguous()


def _ptr(t):
    return t.data_ptr() if t is not None else None


class ReprojectionResidual(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pose_delta, ext_delta, X, pose_qt, ext_qt, K, obs):
        dt = X.dtype
        n = X.shape[0]
        pose_qt = _check(pose_qt, "pose_qt", (7,), dt)
        ext_qt = _check(ext_qt, "ext_qt", (7,), dt)
        X = _check(X, "X", (3,), dt)
        K = _check(K, "K", (4,), dt)
        obs = _check(obs, "obs", (2,), dt)
        pose_delta = _check(pose_delta, "pose_delta", (6,), dt)
        ext_delta = _check(ext_delta, "ext_delta", (6,), dt)
        res = torch.empty((n, 2), dtype=dt, device=X.device)
        stream = torch.cuda.current_stream(X.device).cuda_stream
        N.check(N.lib().mcba_reproj_forward(1 if dt == torch.float64 else 0, n, _ptr(pose_qt), _ptr(ext_qt),
                                            _ptr(pose_delta), _ptr(ext_delta), _ptr(X), _ptr(K), _ptr(obs),
                                            _ptr(res), stream))
        ctx.save_for_backward(pose_delta, ext_delta, X, pose_qt, ext_qt, K)
        return res

    @staticmethod
    def backward(ctx, grad_res):
        pose_delta, ext_delta, X, pose_qt, ext_qt, K = ctx.saved_tensors
        dt = X.dtype
        n = X.shape[0]
        g = grad_res.contiguous()
        gp = torch.empty((n, 6), dtype=dt, device=X.device) if ctx.needs_input_grad[0] else None
        ge = torch.empty((n, 6), dtype=dt, device=X.device) if ctx.needs_input_grad[1] else None
        gx = torch.empty((n, 3), dtype=dt, device=X.device) if ctx.needs_input_grad[2] else None
        stream = torch.cuda.current_stream(X.device).cuda_stream
        N.check(N.lib().mcba_reproj_backward(1 if dt == torch.float64 else 0, n, _ptr(pose_qt), _ptr(ext_qt),
                                             _ptr(pose_delta), _ptr(ext_delta), _ptr(X), _ptr(K), _ptr(g),
                                             _ptr(gp), _ptr(ge), _ptr(gx), None, None, None, stream))
        return gp, ge, gx, None, None, None, None


def reprojection_residual(pose_qt, ext_qt, X, K, obs, pose_delta=None, ext_delta=None):
    """Residuals [n, 2]; differentiable w.r.t. pose_delta, ext_delta and X."""
    n = X.shape[0]
    if pose_delta is None:
        pose_delta = torch.zeros((n, 6), dtype=X.dtype, device=X.device)
    if ext_delta is None:
        ext_delta = torch.zeros((n, 6), dtype=X.dtype, device=X.device)
    return ReprojectionResidual.apply(pose_delta, ext_delta, X, pose_qt, ext_qt, K, obs)


def jacobians(pose_qt, ext_qt, X, K, pose_delta=None, ext_delta=None):
    """Per-edge Jacobians (J_pose [n,2,6], J_ext [n,2,6], J_X [n,2,3]) of the residual."""
    dt = X.dtype
    n = X.shape[0]
    Jp = torch.empty((n, 2, 6), dtype=dt, device=X.device)
    Je = torch.empty((n, 2, 6), dtype=dt, device=X.device)
    Jx = torch.empty((n, 2, 3), dtype=dt, device=X.device)
    pose_qt = _check(pose_qt, "pose_qt", (7,), dt)
    ext_qt = _check(ext_qt, "ext_qt", (7,), dt)
    X = _check(X, "X", (3,), dt)
    K = _check(K, "K", (4,), dt)
    stream = torch.cuda.current_stream(X.device).cuda_stream
    N.check(N.lib().mcba_reproj_backward(1 if dt == torch.float64 else 0, n, _ptr(pose_qt), _ptr(ext_qt),
                                         _ptr(pose_delta), _ptr(ext_delta), _ptr(X), _ptr(K), None, None, None,
                                         None, _ptr(Jp), _ptr(Je), _ptr(Jx), stream))
    return Jp, Je, Jx
