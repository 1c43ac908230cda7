// mcba_reproj.cu -- reprojection residual of EdgeSE3XYZ2Camera as a pair of
// device-pointer entry points (forward residual, backward vector-Jacobian
// product), the kernels behind the autograd harness.
//
//   r = obs - pi(T_cb * T_bw * X)          include/OptimizeTypes.hpp:80-86
//   J_pose = -Jpi R_cb [-[P_b]x | I]        include/OptimizeTypes.hpp:94-113
//   J_X    = -Jpi R_cb R_bw
//   J_ext  = -Jpi [-[P_c]x | I]             (the rig extrinsic, not in the
//                                            reference: T_cb is constant there)
// Perturbations are left-multiplicative, rotation first (g2o's SE3Quat::exp
// convention): T <- exp(delta) * T.  Optional deltas are applied before the
// projection so that finite differences can be taken through the same code.

#include <cuda_runtime.h>

#include <cstdint>

#include "mcba.h"

namespace {

template <typename R>
__device__ __forceinline__ void rot_of(const R* q, R* M) {
  const R x = q[0], y = q[1], z = q[2], w = q[3];
  const R n = sqrt(x * x + y * y + z * z + w * w);
  const R a = x / n, b = y / n, c = z / n, d = w / n;
  M[0] = 1 - 2 * (b * b + c * c);
  M[1] = 2 * (a * b - c * d);
  M[2] = 2 * (a * c + b * d);
  M[3] = 2 * (a * b + c * d);
  M[4] = 1 - 2 * (a * a + c * c);
  M[5] = 2 * (b * c - a * d);
  M[6] = 2 * (a * c - b * d);
  M[7] = 2 * (b * c + a * d);
  M[8] = 1 - 2 * (a * a + b * b);
}

// exp(delta) as rotation matrix + translation (SE3Quat::exp, se3quat.h:218-257).
template <typename R>
__device__ __forceinline__ void exp_se3(const R* u, R* Rm, R* t) {
  const R w0 = u[0], w1 = u[1], w2 = u[2];
  const R th = sqrt(w0 * w0 + w1 * w1 + w2 * w2);
  const R O[9] = {0, -w2, w1, w2, 0, -w0, -w1, w0, 0};
  R O2[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) O2[3 * i + j] = O[3 * i] * O[j] + O[3 * i + 1] * O[3 + j] + O[3 * i + 2] * O[6 + j];
  R a, b, c;
  if (th < R(1e-5)) {
    a = 1;
    b = R(0.5);
    c = R(1.0 / 6.0);
  } else {
    a = sin(th) / th;
    b = (1 - cos(th)) / (th * th);
    c = (th - sin(th)) / (th * th * th);
  }
  R V[9];
  for (int i = 0; i < 9; ++i) {
    const R I = (i % 4 == 0) ? R(1) : R(0);
    Rm[i] = I + a * O[i] + b * O2[i];
    V[i] = I + b * O[i] + c * O2[i];
  }
  for (int i = 0; i < 3; ++i) t[i] = V[3 * i] * u[3] + V[3 * i + 1] * u[4] + V[3 * i + 2] * u[5];
}

// Pose as (R, t), optionally left-perturbed.
template <typename R>
__device__ __forceinline__ void load_pose(const R* qt, const R* delta, R* Rm, R* t) {
  R R0[9];
  rot_of(qt, R0);
  const R t0[3] = {qt[4], qt[5], qt[6]};
  if (!delta) {
    for (int i = 0; i < 9; ++i) Rm[i] = R0[i];
    for (int i = 0; i < 3; ++i) t[i] = t0[i];
    return;
  }
  R Re[9], te[3];
  exp_se3(delta, Re, te);
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) Rm[3 * i + j] = Re[3 * i] * R0[j] + Re[3 * i + 1] * R0[3 + j] + Re[3 * i + 2] * R0[6 + j];
    t[i] = Re[3 * i] * t0[0] + Re[3 * i + 1] * t0[1] + Re[3 * i + 2] * t0[2] + te[i];
  }
}

template <typename R>
struct Geo {
  R Rb[9], Rc[9];
  R Pb[3], Pc[3];
};

template <typename R>
__device__ __forceinline__ void geometry(int64_t i, const R* pose, const R* ext, const R* dp, const R* de, const R* X,
                                         Geo<R>& g) {
  R tb[3], tc[3];
  load_pose(pose + 7 * i, dp ? dp + 6 * i : nullptr, g.Rb, tb);
  load_pose(ext + 7 * i, de ? de + 6 * i : nullptr, g.Rc, tc);
  const R* x = X + 3 * i;
  for (int r = 0; r < 3; ++r) g.Pb[r] = g.Rb[3 * r] * x[0] + g.Rb[3 * r + 1] * x[1] + g.Rb[3 * r + 2] * x[2] + tb[r];
  for (int r = 0; r < 3; ++r)
    g.Pc[r] = g.Rc[3 * r] * g.Pb[0] + g.Rc[3 * r + 1] * g.Pb[1] + g.Rc[3 * r + 2] * g.Pb[2] + tc[r];
}

template <typename R>
__global__ void k_reproj_fwd(int64_t n, const R* pose, const R* ext, const R* dp, const R* de, const R* X,
                             const R* K, const R* obs, R* res) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  Geo<R> g;
  geometry(i, pose, ext, dp, de, X, g);
  const R* k = K + 4 * i;
  res[2 * i] = obs[2 * i] - (k[0] * g.Pc[0] / g.Pc[2] + k[2]);
  res[2 * i + 1] = obs[2 * i + 1] - (k[1] * g.Pc[1] / g.Pc[2] + k[3]);
}

template <typename R>
__global__ void k_reproj_bwd(int64_t n, const R* pose, const R* ext, const R* dp, const R* de, const R* X,
                             const R* K, const R* gres, R* g_pose, R* g_ext, R* g_X, R* J_pose, R* J_ext, R* J_X) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  Geo<R> g;
  geometry(i, pose, ext, dp, de, X, g);
  const R* k = K + 4 * i;
  const R z = g.Pc[2], z2 = z * z;
  // A = -Jpi (2x3)
  const R A[2][3] = {{-k[0] / z, 0, k[0] * g.Pc[0] / z2}, {0, -k[1] / z, k[1] * g.Pc[1] / z2}};
  R M[2][3];  // A R_cb
  for (int r = 0; r < 2; ++r)
    for (int j = 0; j < 3; ++j) M[r][j] = A[r][0] * g.Rc[j] + A[r][1] * g.Rc[3 + j] + A[r][2] * g.Rc[6 + j];
  R Jp[2][6], Je[2][6], Jx[2][3];
  for (int r = 0; r < 2; ++r) {
    Jp[r][0] = g.Pb[1] * M[r][2] - g.Pb[2] * M[r][1];
    Jp[r][1] = g.Pb[2] * M[r][0] - g.Pb[0] * M[r][2];
    Jp[r][2] = g.Pb[0] * M[r][1] - g.Pb[1] * M[r][0];
    Jp[r][3] = M[r][0];
    Jp[r][4] = M[r][1];
    Jp[r][5] = M[r][2];
    Je[r][0] = g.Pc[1] * A[r][2] - g.Pc[2] * A[r][1];
    Je[r][1] = g.Pc[2] * A[r][0] - g.Pc[0] * A[r][2];
    Je[r][2] = g.Pc[0] * A[r][1] - g.Pc[1] * A[r][0];
    Je[r][3] = A[r][0];
    Je[r][4] = A[r][1];
    Je[r][5] = A[r][2];
    for (int j = 0; j < 3; ++j) Jx[r][j] = M[r][0] * g.Rb[j] + M[r][1] * g.Rb[3 + j] + M[r][2] * g.Rb[6 + j];
  }
  const R g0 = gres ? gres[2 * i] : R(0), g1 = gres ? gres[2 * i + 1] : R(0);
  if (g_pose)
    for (int j = 0; j < 6; ++j) g_pose[6 * i + j] = Jp[0][j] * g0 + Jp[1][j] * g1;
  if (g_ext)
    for (int j = 0; j < 6; ++j) g_ext[6 * i + j] = Je[0][j] * g0 + Je[1][j] * g1;
  if (g_X)
    for (int j = 0; j < 3; ++j) g_X[3 * i + j] = Jx[0][j] * g0 + Jx[1][j] * g1;
  if (J_pose)
    for (int r = 0; r < 2; ++r)
      for (int j = 0; j < 6; ++j) J_pose[12 * i + 6 * r + j] = Jp[r][j];
  if (J_ext)
    for (int r = 0; r < 2; ++r)
      for (int j = 0; j < 6; ++j) J_ext[12 * i + 6 * r + j] = Je[r][j];
  if (J_X)
    for (int r = 0; r < 2; ++r)
      for (int j = 0; j < 3; ++j) J_X[6 * i + 3 * r + j] = Jx[r][j];
}

int launch_status(cudaError_t e) { return e == cudaSuccess ? MCBA_OK : MCBA_ERR_CUDA; }

}  // namespace

extern "C" int mcba_reproj_forward(int32_t dbl, int64_t n, const void* pose_qt, const void* ext_qt,
                                   const void* pose_delta, const void* ext_delta, const void* X, const void* K,
                                   const void* obs, void* res, void* stream) {
  if (n < 0) return MCBA_ERR_INVALID;
  if (n == 0) return MCBA_OK;
  if (!pose_qt || !ext_qt || !X || !K || !obs || !res) return MCBA_ERR_INVALID;
  const int threads = 256;
  const unsigned blocks = (unsigned)((n + threads - 1) / threads);
  cudaStream_t st = (cudaStream_t)stream;
  if (dbl)
    k_reproj_fwd<double><<<blocks, threads, 0, st>>>(n, (const double*)pose_qt, (const double*)ext_qt,
                                                     (const double*)pose_delta, (const double*)ext_delta,
                                                     (const double*)X, (const double*)K, (const double*)obs,
                                                     (double*)res);
  else
    k_reproj_fwd<float><<<blocks, threads, 0, st>>>(n, (const float*)pose_qt, (const float*)ext_qt,
                                                    (const float*)pose_delta, (const float*)ext_delta,
                                                    (const float*)X, (const float*)K, (const float*)obs, (float*)res);
  return launch_status(cudaGetLastError());
}

extern "C" int mcba_reproj_backward(int32_t dbl, int64_t n, const void* pose_qt, const void* ext_qt,
                                    const void* pose_delta, const void* ext_delta, const void* X, const void* K,
                                    const void* grad_res, void* g_pose, void* g_ext, void* g_X, void* J_pose,
                                    void* J_ext, void* J_X, void* stream) {
  if (n < 0) return MCBA_ERR_INVALID;
  if (n == 0) return MCBA_OK;
  if (!pose_qt || !ext_qt || !X || !K) return MCBA_ERR_INVALID;
  if ((g_pose || g_ext || g_X) && !grad_res) return MCBA_ERR_INVALID;
  const int threads = 256;
  const unsigned blocks = (unsigned)((n + threads - 1) / threads);
  cudaStream_t st = (cudaStream_t)stream;
  if (dbl)
    k_reproj_bwd<double><<<blocks, threads, 0, st>>>(
        n, (const double*)pose_qt, (const double*)ext_qt, (const double*)pose_delta, (const double*)ext_delta,
        (const double*)X, (const double*)K, (const double*)grad_res, (double*)g_pose, (double*)g_ext, (double*)g_X,
        (double*)J_pose, (double*)J_ext, (double*)J_X);
  else
    k_reproj_bwd<float><<<blocks, threads, 0, st>>>(
        n, (const float*)pose_qt, (const float*)ext_qt, (const float*)pose_delta, (const float*)ext_delta,
        (const float*)X, (const float*)K, (const float*)grad_res, (float*)g_pose, (float*)g_ext, (float*)g_X,
        (float*)J_pose, (float*)J_ext, (float*)J_X);
  return launch_status(cudaGetLastError());
}
