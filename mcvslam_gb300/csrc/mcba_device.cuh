// mcba_device.cuh -- device-side math shared by the solver kernels:
// SE3 helpers, the three reprojection edges of MCVSLAM's OptimizeTypes, the
// Huber kernel and warp/block reductions.  Templated on the linearisation
// real type R (double for the FP64 plain solver, float for mixed precision).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "mcba_internal.h"

namespace mcba {
namespace dev {

// Pose data used by the edge kernels, derived from the quaternion state.
struct PoseLinD {
  double R[9];  // R_body_world (row-major)
  double t[3];  // t_body_world
};
struct PoseLinF {
  float R[9];   // R_body_world
  float c[3];   // body centre in the world, -R^T t (points are taken relative to it)
};
struct CamD {
  double K[4];   // fx fy cx cy (float parameters promoted)
  double bf;
  double R[9];   // R_cam_body
  double t[3];
};
struct CamF {
  float K[4];
  float bf;
  float R[9];
  float t[3];
};

// 1/sqrt(d) for a positive double: FP32 estimate refined by two
// Newton-Raphson steps y <- y (3 - d y^2) / 2 (quadratic convergence, from
// ~2^-22 to full precision).  GB300 has little FP64 throughput, so chains of
// FP64 square roots and divisions are replaced by this and multiplications.
__device__ __forceinline__ double rsqrt_newton(double d) {
  if (!(d > 1e-36 && d < 1e36)) return 1.0 / sqrt(d);
  double y = (double)rsqrtf((float)d);
  const double hd = 0.5 * d;
  y = y * (1.5 - hd * y * y);
  y = y * (1.5 - hd * y * y);
  return y;
}

// Unit quaternion (x y z w) -> row-major rotation matrix.
__device__ __forceinline__ void quat_to_R(const double* q, double* R) {
  const double x = q[0], y = q[1], z = q[2], w = q[3];
  const double tx = 2 * x, ty = 2 * y, tz = 2 * z;
  const double twx = tx * w, twy = ty * w, twz = tz * w;
  const double txx = tx * x, txy = ty * x, txz = tz * x;
  const double tyy = ty * y, tyz = tz * y, tzz = tz * z;
  R[0] = 1 - (tyy + tzz);
  R[1] = txy - twz;
  R[2] = txz + twy;
  R[3] = txy + twz;
  R[4] = 1 - (txx + tzz);
  R[5] = tyz - twx;
  R[6] = txz - twy;
  R[7] = tyz + twx;
  R[8] = 1 - (txx + tyy);
}

// Shoemake's rotation-matrix -> quaternion, then w >= 0 and unit norm
// (SE3Quat(R, t), types/slam3d/se3quat.h:53-55,280-285).
__device__ __forceinline__ void R_to_quat(const double* R, double* q) {
  double x, y, z, w;
  const double tr = R[0] + R[4] + R[8];
  if (tr > 0) {
    const double a = tr + 1.0, ys = rsqrt_newton(a);
    w = 0.5 * (a * ys);
    const double s = 0.5 * ys;
    x = (R[7] - R[5]) * s;
    y = (R[2] - R[6]) * s;
    z = (R[3] - R[1]) * s;
  } else {
    int i = 0;
    if (R[4] > R[0]) i = 1;
    if (R[8] > R[4 * i]) i = 2;
    const int j = (i + 1) % 3, k = (j + 1) % 3;
    const double a = R[4 * i] - R[4 * j] - R[4 * k] + 1.0, ys = rsqrt_newton(a);
    double v[3];
    v[i] = 0.5 * (a * ys);
    const double s = 0.5 * ys;
    w = (R[3 * k + j] - R[3 * j + k]) * s;
    v[j] = (R[3 * j + i] + R[3 * i + j]) * s;
    v[k] = (R[3 * k + i] + R[3 * i + k]) * s;
    x = v[0];
    y = v[1];
    z = v[2];
  }
  if (w < 0) {
    x = -x;
    y = -y;
    z = -z;
    w = -w;
  }
  const double in = rsqrt_newton(x * x + y * y + z * z + w * w);
  q[0] = x * in;
  q[1] = y * in;
  q[2] = z * in;
  q[3] = w * in;
}

// Rotate v by the unit quaternion q: v + w*uv + q x uv with uv = 2 q x v.
__device__ __forceinline__ void quat_rotate(const double* q, const double* v, double* o) {
  double uv0 = q[1] * v[2] - q[2] * v[1], uv1 = q[2] * v[0] - q[0] * v[2], uv2 = q[0] * v[1] - q[1] * v[0];
  uv0 += uv0;
  uv1 += uv1;
  uv2 += uv2;
  o[0] = v[0] + q[3] * uv0 + (q[1] * uv2 - q[2] * uv1);
  o[1] = v[1] + q[3] * uv1 + (q[2] * uv0 - q[0] * uv2);
  o[2] = v[2] + q[3] * uv2 + (q[0] * uv1 - q[1] * uv0);
}

// SE3Quat::exp (types/slam3d/se3quat.h:218-257) followed by the left
// composition of VertexSE3Expmap::oplusImpl (types_six_dof_expmap.h:98-101):
// T <- exp(u) * T, with the quaternion product, t' = t_exp + r_exp * t, and
// normalizeRotation.  qt = x y z w tx ty tz.
__device__ __forceinline__ void se3_exp_left(const double* u, const double* qt_in, double* qt_out) {
  const double w0 = u[0], w1 = u[1], w2 = u[2];
  const double th2 = w0 * w0 + w1 * w1 + w2 * w2;
  // Omega = skew(w), Omega^2
  const double O[9] = {0, -w2, w1, w2, 0, -w0, -w1, w0, 0};
  double O2[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) O2[3 * i + j] = O[3 * i] * O[j] + O[3 * i + 1] * O[3 + j] + O[3 * i + 2] * O[6 + j];
  double vb, vc, qe[4];
  if (th2 < 1e-10) {  // theta < 1e-5: R = I + Omega + Omega^2 / 2, then Quaternion(R)
    vb = 0.5;
    vc = 1.0 / 6.0;
    double R[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) R[i] = ((i % 4 == 0) ? 1.0 : 0.0) + O[i] + 0.5 * O2[i];
    R_to_quat(R, qe);
  } else {
    // The quaternion of the Rodrigues rotation R = I + sin(t)/t Omega +
    // (1 - cos(t))/t^2 Omega^2 is (sin(t/2) w/t, cos(t/2)), which is what
    // Quaternion(R) returns for it up to rounding, without R's square root
    // and normalisation on the dependency chain.  V takes sin(t) =
    // 2 sin(t/2) cos(t/2) and 1 - cos(t) = 2 sin^2(t/2).
    const double inv = rsqrt_newton(th2), theta = th2 * inv;
    double sh, ch;
    sincos(0.5 * theta, &sh, &ch);
    const double k = sh * inv;
    qe[0] = w0 * k;
    qe[1] = w1 * k;
    qe[2] = w2 * k;
    qe[3] = ch;
    const double s = 2.0 * sh * ch;
    vb = 2.0 * sh * sh * (inv * inv);
    vc = (theta - s) * (inv * inv * inv);
  }
  double V[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) V[i] = ((i % 4 == 0) ? 1.0 : 0.0) + vb * O[i] + vc * O2[i];
  const double te[3] = {V[0] * u[3] + V[1] * u[4] + V[2] * u[5], V[3] * u[3] + V[4] * u[4] + V[5] * u[5],
                        V[6] * u[3] + V[7] * u[4] + V[8] * u[5]};
  // exp(u) * T
  double rt[3];
  quat_rotate(qe, qt_in + 4, rt);
  const double* q2 = qt_in;
  double x = qe[3] * q2[0] + qe[0] * q2[3] + qe[1] * q2[2] - qe[2] * q2[1];
  double y = qe[3] * q2[1] + qe[1] * q2[3] + qe[2] * q2[0] - qe[0] * q2[2];
  double z = qe[3] * q2[2] + qe[2] * q2[3] + qe[0] * q2[1] - qe[1] * q2[0];
  double w = qe[3] * q2[3] - qe[0] * q2[0] - qe[1] * q2[1] - qe[2] * q2[2];
  if (w < 0) {
    x = -x;
    y = -y;
    z = -z;
    w = -w;
  }
  const double in = rsqrt_newton(x * x + y * y + z * z + w * w);
  qt_out[0] = x * in;
  qt_out[1] = y * in;
  qt_out[2] = z * in;
  qt_out[3] = w * in;
  qt_out[4] = te[0] + rt[0];
  qt_out[5] = te[1] + rt[1];
  qt_out[6] = te[2] + rt[2];
}

// ------------------------------------------------------------ edges --
template <typename R>
struct EdgeLin {
  R e[3];
  R chi2;
  R w;    // rho' * info (robust information scale)
  R s;    // rho'
  R Jl[3][3];
  R Jp[3][6];
};

// Huber rho' (robust_kernel_impl.cpp:65-78): 1 inside delta^2, delta/sqrt(e2) outside.
template <typename R>
__device__ __forceinline__ R huber_d1(R e2, R delta) {
  const R dsqr = delta * delta;
  return (e2 <= dsqr) ? R(1) : delta / sqrt(e2);
}
template <typename R>
__device__ __forceinline__ R huber_rho(R e2, R delta) {
  const R dsqr = delta * delta;
  return (e2 <= dsqr) ? e2 : R(2) * sqrt(e2) * delta - dsqr;
}

struct StateView {
  const PoseLinD* pd;
  const PoseLinF* pf;
  const double* Xd;  // [P+U][3]
  const float4* Xf;  // [P+U]
  const CamD* cd;
  const CamF* cf;
};

// Point in the camera frame (and, for mono/unary edges, in the body frame).
__device__ __forceinline__ void transform(const EdgeRec& r, const StateView& v, double* Pb, double* Pc) {
  const PoseLinD& P = v.pd[r.pose];
  const double* X = v.Xd + 3 * (size_t)r.point;
  const double x0 = X[0], x1 = X[1], x2 = X[2];
  const double b0 = P.R[0] * x0 + P.R[1] * x1 + P.R[2] * x2 + P.t[0];
  const double b1 = P.R[3] * x0 + P.R[4] * x1 + P.R[5] * x2 + P.t[1];
  const double b2 = P.R[6] * x0 + P.R[7] * x1 + P.R[8] * x2 + P.t[2];
  Pb[0] = b0;
  Pb[1] = b1;
  Pb[2] = b2;
  if (r.type == MCBA_EDGE_STEREO) {
    Pc[0] = b0;
    Pc[1] = b1;
    Pc[2] = b2;
  } else {
    const CamD& C = v.cd[r.cam];
    Pc[0] = C.R[0] * b0 + C.R[1] * b1 + C.R[2] * b2 + C.t[0];
    Pc[1] = C.R[3] * b0 + C.R[4] * b1 + C.R[5] * b2 + C.t[1];
    Pc[2] = C.R[6] * b0 + C.R[7] * b1 + C.R[8] * b2 + C.t[2];
  }
}
__device__ __forceinline__ void transform(const EdgeRec& r, const StateView& v, float* Pb, float* Pc) {
  const PoseLinF& P = v.pf[r.pose];
  const float4 X = v.Xf[r.point];
  const float x0 = X.x - P.c[0], x1 = X.y - P.c[1], x2 = X.z - P.c[2];
  const float b0 = P.R[0] * x0 + P.R[1] * x1 + P.R[2] * x2;
  const float b1 = P.R[3] * x0 + P.R[4] * x1 + P.R[5] * x2;
  const float b2 = P.R[6] * x0 + P.R[7] * x1 + P.R[8] * x2;
  Pb[0] = b0;
  Pb[1] = b1;
  Pb[2] = b2;
  if (r.type == MCBA_EDGE_STEREO) {
    Pc[0] = b0;
    Pc[1] = b1;
    Pc[2] = b2;
  } else {
    const CamF& C = v.cf[r.cam];
    Pc[0] = C.R[0] * b0 + C.R[1] * b1 + C.R[2] * b2 + C.t[0];
    Pc[1] = C.R[3] * b0 + C.R[4] * b1 + C.R[5] * b2 + C.t[1];
    Pc[2] = C.R[6] * b0 + C.R[7] * b1 + C.R[8] * b2 + C.t[2];
  }
}

template <typename R>
struct CamSel;
template <>
struct CamSel<double> {
  __device__ static const CamD& get(const StateView& v, int c) { return v.cd[c]; }
  __device__ static const double* rot(const StateView& v, int p) { return v.pd[p].R; }
};
template <>
struct CamSel<float> {
  __device__ static const CamF& get(const StateView& v, int c) { return v.cf[c]; }
  __device__ static const float* rot(const StateView& v, int p) { return v.pf[p].R; }
};

// Residual and chi2 (computeError + BaseEdge::chi2):
//  mono/unary  e = z - pi(P_cam)                       OptimizeTypes.hpp:29-33,80-86
//  stereo      e = z - (u, v, u - bf*invz), invz float OptimizeTypes.hpp:127-133,144-154
// The stereo projection keeps the reference's float invz and float bf*invz.
template <typename R>
__device__ __forceinline__ void edge_error(const EdgeRec& r, const float* obs, const StateView& v, const R* Pc,
                                           R* e, R& chi2) {
  const auto& C = CamSel<R>::get(v, r.cam);
  const R info = (R)r.info;
  if (r.type == MCBA_EDGE_STEREO) {
    const float invz = (float)(R(1) / Pc[2]);
    const R u = Pc[0] * (R)invz * C.K[0] + C.K[2];
    const R vv = Pc[1] * (R)invz * C.K[1] + C.K[3];
    const float bff = (float)C.bf;
    const R ur = u - (R)__fmul_rn(bff, invz);
    e[0] = (R)obs[0] - u;
    e[1] = (R)obs[1] - vv;
    e[2] = (R)obs[2] - ur;
    chi2 = e[0] * (info * e[0]) + e[1] * (info * e[1]) + e[2] * (info * e[2]);
  } else {
    const R u = C.K[0] * Pc[0] / Pc[2] + C.K[2];
    const R vv = C.K[1] * Pc[1] / Pc[2] + C.K[3];
    e[0] = (R)obs[0] - u;
    e[1] = (R)obs[1] - vv;
    e[2] = R(0);
    chi2 = e[0] * (info * e[0]) + e[1] * (info * e[1]);
  }
}

// Jacobians (linearizeOplus):
//  mono   include/OptimizeTypes.hpp:94-113: J_point = -Jpi R_cw,
//         J_pose = -Jpi R_cb [-[P_b]x | I]
//  unary  include/OptimizeTypes.hpp:40-63: J_pose as above
//  stereo src/OptimizeTypes.cpp:12-58
// Pinhole Jpi: modules/camera/Pinhole.cpp:105-116.
template <typename R>
__device__ __forceinline__ void edge_jac(const EdgeRec& r, const StateView& v, const R* Pb, const R* Pc,
                                         R (&Jl)[3][3], R (&Jp)[3][6]) {
  const auto& C = CamSel<R>::get(v, r.cam);
  const R* Rb = CamSel<R>::rot(v, r.pose);
  if (r.type == MCBA_EDGE_STEREO) {
    const R x = Pc[0], y = Pc[1], z = Pc[2], z_2 = z * z;
    const R fx = C.K[0], fy = C.K[1], bf = C.bf;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      Jl[0][j] = -fx * Rb[j] / z + fx * x * Rb[6 + j] / z_2;
      Jl[1][j] = -fy * Rb[3 + j] / z + fy * y * Rb[6 + j] / z_2;
      Jl[2][j] = Jl[0][j] - bf * Rb[6 + j] / z_2;
    }
    Jp[0][0] = x * y / z_2 * fx;
    Jp[0][1] = -(1 + (x * x / z_2)) * fx;
    Jp[0][2] = y / z * fx;
    Jp[0][3] = R(-1) / z * fx;
    Jp[0][4] = 0;
    Jp[0][5] = x / z_2 * fx;
    Jp[1][0] = (1 + y * y / z_2) * fy;
    Jp[1][1] = -x * y / z_2 * fy;
    Jp[1][2] = -x / z * fy;
    Jp[1][3] = 0;
    Jp[1][4] = R(-1) / z * fy;
    Jp[1][5] = y / z_2 * fy;
    Jp[2][0] = Jp[0][0] - bf * y / z_2;
    Jp[2][1] = Jp[0][1] + bf * x / z_2;
    Jp[2][2] = Jp[0][2];
    Jp[2][3] = Jp[0][3];
    Jp[2][4] = 0;
    Jp[2][5] = Jp[0][5] - bf / z_2;
    return;
  }
  const R z = Pc[2];
  const R z2 = z * z;
  // -Jpi rows: [-fx/z, 0, fx x/z^2], [0, -fy/z, fy y/z^2]
  const R a00 = -C.K[0] / z, a02 = C.K[0] * Pc[0] / z2;
  const R a11 = -C.K[1] / z, a12 = C.K[1] * Pc[1] / z2;
  R M[2][3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    M[0][j] = a00 * C.R[j] + a02 * C.R[6 + j];
    M[1][j] = a11 * C.R[3 + j] + a12 * C.R[6 + j];
  }
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    // rotation part: M * (-[Pb]x) = Pb x M
    Jp[k][0] = Pb[1] * M[k][2] - Pb[2] * M[k][1];
    Jp[k][1] = Pb[2] * M[k][0] - Pb[0] * M[k][2];
    Jp[k][2] = Pb[0] * M[k][1] - Pb[1] * M[k][0];
    Jp[k][3] = M[k][0];
    Jp[k][4] = M[k][1];
    Jp[k][5] = M[k][2];
#pragma unroll
    for (int j = 0; j < 3; ++j) Jl[k][j] = M[k][0] * Rb[j] + M[k][1] * Rb[3 + j] + M[k][2] * Rb[6 + j];
  }
#pragma unroll
  for (int j = 0; j < 6; ++j) Jp[2][j] = 0;
#pragma unroll
  for (int j = 0; j < 3; ++j) Jl[2][j] = 0;
}

// ------------------------------------------------------ reductions --
// Accumulator of the linearisation real type.  FP64: a plain double.  FP32:
// a float-float pair updated with Knuth's TwoSum, so that long FP32 sums
// (thousands of edges per pose, of pairs per reduced-camera block) keep the
// information that cancels in the Schur complement; all arithmetic stays FP32.
template <typename R>
struct Acc;
template <>
struct Acc<double> {
  double v;
  __device__ __forceinline__ void zero() { v = 0.0; }
  __device__ __forceinline__ void add(double x) { v += x; }
  __device__ __forceinline__ void add(const Acc& o) { v += o.v; }
  __device__ __forceinline__ double value() const { return v; }
  __device__ __forceinline__ Acc shfl_xor(int m) const {
    Acc r;
    r.v = __shfl_xor_sync(0xffffffffu, v, m);
    return r;
  }
};
template <>
struct Acc<float> {
  float hi, lo;
  __device__ __forceinline__ void zero() { hi = lo = 0.f; }
  __device__ __forceinline__ void add(float x) {
    const float s = __fadd_rn(hi, x);
    const float bb = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(x, bb));
    hi = s;
    lo = __fadd_rn(lo, err);
  }
  __device__ __forceinline__ void add(const Acc& o) {
    const float s = __fadd_rn(hi, o.hi);
    const float bb = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(o.hi, bb));
    hi = s;
    lo = __fadd_rn(__fadd_rn(lo, o.lo), err);
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
  __device__ __forceinline__ Acc shfl_xor(int m) const {
    Acc r;
    r.hi = __shfl_xor_sync(0xffffffffu, hi, m);
    r.lo = __shfl_xor_sync(0xffffffffu, lo, m);
    return r;
  }
};

// Reduce-scatter of 32 per-lane accumulators: afterwards lane l holds the
// warp sum of slot l (recursive halving, 31 exchanges per lane).
template <typename A>
__device__ __forceinline__ A warp_reduce_scatter32_acc(A (&v)[32]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int s = 16; s >= 1; s >>= 1) {
    const bool upper = (lane & s) != 0;
#pragma unroll
    for (int i = 0; i < s; ++i) {
      const A send = upper ? v[i] : v[i + s];
      A keep = upper ? v[i + s] : v[i];
      keep.add(send.shfl_xor(s));
      v[i] = keep;
    }
  }
  return v[0];
}

template <typename A>
__device__ __forceinline__ A warp_sum_acc(A x) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) x.add(x.shfl_xor(o));
  return x;
}

// Reduce-scatter of 32 per-lane values: afterwards lane l holds the warp sum
// of slot l (recursive halving, 31 shuffles per lane).
template <typename T>
__device__ __forceinline__ T warp_reduce_scatter32(T (&v)[32]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int s = 16; s >= 1; s >>= 1) {
    const bool upper = (lane & s) != 0;
#pragma unroll
    for (int i = 0; i < s; ++i) {
      const T send = upper ? v[i] : v[i + s];
      const T keep = upper ? v[i + s] : v[i];
      const T recv = __shfl_xor_sync(0xffffffffu, send, s);
      v[i] = keep + recv;
    }
  }
  return v[0];
}

template <typename T>
__device__ __forceinline__ T warp_sum(T x) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

template <typename T>
__device__ __forceinline__ T warp_max(T x) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) x = max(x, __shfl_xor_sync(0xffffffffu, x, o));
  return x;
}

// Deterministic block sum (fixed tree) of one value per thread; every
// thread gets the result.  blockDim.x must be a multiple of 32, <= 1024.
template <typename T>
__device__ __forceinline__ T block_sum(T x, T* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  x = warp_sum(x);
  __syncthreads();
  if (lane == 0) sh[wid] = x;
  __syncthreads();
  T r = (lane < nw) ? sh[lane] : T(0);
  r = warp_sum(r);
  return r;
}

}  // namespace dev
}  // namespace mcba
