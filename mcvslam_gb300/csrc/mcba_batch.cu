// mcba_batch.cu -- many independent pose-only optimisations in one launch.
//
// PoseEstimation::PoseOptimization (src/PoseEstimation.cpp:48-130) optimises
// one frame's body pose against fixed map points: 4 rounds of g2o LM
// (15 iterations each in the reference), after each round every remaining
// edge with chi2 >= 5.991 is set to level 1 (never re-admitted), the robust
// kernels are removed after round 2, and the loop stops early when fewer than
// 10 edges remain.  With one free pose and all points fixed, g2o's Schur
// solver degenerates to the 6x6 pose block, so each problem is small.
//
// Here a persistent kernel takes problems from an atomic work queue, one CTA
// per problem: the CTA's threads stream the problem's edges (residual, Huber
// weight, 2x6 Jacobian, J^T W J and J^T W e in the linearisation real type R,
// compensated accumulation for FP32), thread 0 runs the LM control, the 6x6
// LL^T solve and the SE3 retraction in FP64.  The whole batch is one graph
// launch (queue reset + kernel); no host round trip per problem or per trial.

#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "mcba.h"
#include "mcba_device.cuh"

namespace mcba {
namespace {
using namespace dev;

struct BatchArgs {
  int n;                    // problems
  const int* edge_begin;    // [n+1]
  const int* cam;           // [E]
  const float* obs;         // [E][2]
  const float* Xw;          // [E][3]
  const float* info;        // [E]
  const float* delta;       // [E]
  const CamD* cd;
  const CamF* cf;
  double* qt;               // [n][8] in/out
  uint8_t* level;           // [E] out
  int* inliers;             // [n] out
  int* queue;               // work counter
  int rounds, iters, drop_round, max_trials;
  float thr;
  double tau;
};

template <typename R>
struct PoseR;
template <>
struct PoseR<double> {
  double R[9], t[3];
};
template <>
struct PoseR<float> {
  float R[9], c[3];
};

__device__ void pose_of(const double* qt, PoseR<double>& P) {
  quat_to_R(qt, P.R);
  P.t[0] = qt[4];
  P.t[1] = qt[5];
  P.t[2] = qt[6];
}
__device__ void pose_of(const double* qt, PoseR<float>& P) {
  double Rm[9];
  quat_to_R(qt, Rm);
  for (int k = 0; k < 9; ++k) P.R[k] = (float)Rm[k];
  for (int k = 0; k < 3; ++k) P.c[k] = (float)(-(Rm[k] * qt[4] + Rm[3 + k] * qt[5] + Rm[6 + k] * qt[6]));
}

__device__ __forceinline__ const CamD& cam_of(const BatchArgs& a, int c, double) { return a.cd[c]; }
__device__ __forceinline__ const CamF& cam_of(const BatchArgs& a, int c, float) { return a.cf[c]; }

// Point in body and camera frames for a unary edge.
__device__ __forceinline__ void xform(const PoseR<double>& P, const CamD& C, const float* X, double* Pb, double* Pc) {
  const double x0 = X[0], x1 = X[1], x2 = X[2];
  for (int r = 0; r < 3; ++r) Pb[r] = P.R[3 * r] * x0 + P.R[3 * r + 1] * x1 + P.R[3 * r + 2] * x2 + P.t[r];
  for (int r = 0; r < 3; ++r) Pc[r] = C.R[3 * r] * Pb[0] + C.R[3 * r + 1] * Pb[1] + C.R[3 * r + 2] * Pb[2] + C.t[r];
}
__device__ __forceinline__ void xform(const PoseR<float>& P, const CamF& C, const float* X, float* Pb, float* Pc) {
  const float x0 = X[0] - P.c[0], x1 = X[1] - P.c[1], x2 = X[2] - P.c[2];
  for (int r = 0; r < 3; ++r) Pb[r] = P.R[3 * r] * x0 + P.R[3 * r + 1] * x1 + P.R[3 * r + 2] * x2;
  for (int r = 0; r < 3; ++r) Pc[r] = C.R[3 * r] * Pb[0] + C.R[3 * r + 1] * Pb[1] + C.R[3 * r + 2] * Pb[2] + C.t[r];
}

template <typename R, typename Cm>
__device__ __forceinline__ R chi2_of(const Cm& C, const R* Pc, const float* obs, float info, R* e) {
  const R u = C.K[0] * Pc[0] / Pc[2] + C.K[2];
  const R v = C.K[1] * Pc[1] / Pc[2] + C.K[3];
  e[0] = (R)obs[0] - u;
  e[1] = (R)obs[1] - v;
  const R w = (R)info;
  return e[0] * (w * e[0]) + e[1] * (w * e[1]);
}

// 6x6 SPD solve (H + lambda I) x = b by LL^T; false on a non-positive pivot.
__device__ bool solve6(const double* H, double lam, const double* b, double* x) {
  double L[36];
  for (int i = 0; i < 36; ++i) L[i] = H[i];
  for (int i = 0; i < 6; ++i) L[7 * i] += lam;
  double rd[6];
  bool ok = true;
  for (int j = 0; j < 6; ++j) {
    double d = L[7 * j];
    for (int k = 0; k < j; ++k) d -= L[6 * j + k] * L[6 * j + k];
    if (d <= 0.0) ok = false;
    const double y = rsqrt_newton(d);
    L[7 * j] = d * y;
    rd[j] = y;
    for (int i = j + 1; i < 6; ++i) {
      double s = L[6 * i + j];
      for (int k = 0; k < j; ++k) s -= L[6 * i + k] * L[6 * j + k];
      L[6 * i + j] = s * y;
    }
  }
  double z[6];
  for (int i = 0; i < 6; ++i) {
    double s = b[i];
    for (int k = 0; k < i; ++k) s -= L[6 * i + k] * z[k];
    z[i] = s * rd[i];
  }
  for (int i = 5; i >= 0; --i) {
    double s = z[i];
    for (int k = i + 1; k < 6; ++k) s -= L[6 * k + i] * x[k];
    x[i] = s * rd[i];
  }
  return ok;
}

template <typename R, int T>
struct BlockRed {
  // per-warp partials of 27 quadratic-form slots + cost
  Acc<R> part[T / 32][28];
};

template <typename R, int T>
__global__ void __launch_bounds__(T) k_pose_batch(BatchArgs a) {
  __shared__ double s_qt[8], s_cand[8];
  __shared__ PoseR<R> s_pose, s_pcand;
  __shared__ double s_H[36], s_b[6], s_x[6];
  __shared__ double s_red[T / 32];
  __shared__ BlockRed<R, T> red;
  __shared__ int s_prob, s_nact, s_stop, s_flag_more, s_solve_ok;
  __shared__ double s_lambda, s_ni, s_chi;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;

  for (;;) {
    if (tid == 0) s_prob = atomicAdd(a.queue, 1);
    __syncthreads();
    const int p = s_prob;
    if (p >= a.n) return;
    const int e0 = a.edge_begin[p], e1 = a.edge_begin[p + 1];
    const int nInitial = e1 - e0;
    for (int e = e0 + tid; e < e1; e += T) a.level[e] = 0;
    if (tid < 7) s_qt[tid] = a.qt[8 * (size_t)p + tid];
    __syncthreads();
    if (nInitial < 3) {
      if (tid == 0) a.inliers[p] = 0;
      __syncthreads();
      continue;
    }
    int nBad = 0;
    for (int round = 0; round < a.rounds; ++round) {
      const bool robust = round <= a.drop_round;
      // ---- optimize(iters) on the level-0 edges
      if (tid == 0) pose_of(s_qt, s_pose);
      __syncthreads();
      int nact = 0;
      for (int e = e0 + tid; e < e1; e += T) nact += a.level[e] == 0;
      {
        for (int o = 16; o >= 1; o >>= 1) nact += __shfl_xor_sync(0xffffffffu, nact, o);
        if (lane == 0) s_red[wid] = nact;
        __syncthreads();
        if (tid == 0) {
          int t = 0;
          for (int w = 0; w < T / 32; ++w) t += (int)s_red[w];
          s_nact = t;
        }
        __syncthreads();
      }
      if (s_nact > 0) {
        if (tid == 0) {
          s_stop = 0;
          s_ni = 2.0;
        }
        for (int it = 0; it < a.iters; ++it) {
          __syncthreads();
          if (s_stop) break;
          // linearise at the current pose: H, b, cost
          Acc<R> acc[28];
#pragma unroll
          for (int k = 0; k < 28; ++k) acc[k].zero();
          for (int e = e0 + tid; e < e1; e += T) {
            if (a.level[e]) continue;
            const auto& C = cam_of(a, a.cam[e], R(0));
            R Pb[3], Pc[3], ev[2];
            xform(s_pose, C, a.Xw + 3 * (size_t)e, Pb, Pc);
            const R chi2 = chi2_of<R>(C, Pc, a.obs + 2 * (size_t)e, a.info[e], ev);
            const R dl = (R)a.delta[e];
            R s = R(1), rho = chi2;
            if (robust && dl > R(0)) {
              s = huber_d1<R>(chi2, dl);
              rho = huber_rho<R>(chi2, dl);
            }
            const R w = s * (R)a.info[e];
            const R z = Pc[2], z2 = z * z;
            const R a00 = -C.K[0] / z, a02 = C.K[0] * Pc[0] / z2, a11 = -C.K[1] / z, a12 = C.K[1] * Pc[1] / z2;
            R M[2][3], J[2][6];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
              M[0][j] = a00 * C.R[j] + a02 * C.R[6 + j];
              M[1][j] = a11 * C.R[3 + j] + a12 * C.R[6 + j];
            }
#pragma unroll
            for (int k = 0; k < 2; ++k) {
              J[k][0] = Pb[1] * M[k][2] - Pb[2] * M[k][1];
              J[k][1] = Pb[2] * M[k][0] - Pb[0] * M[k][2];
              J[k][2] = Pb[0] * M[k][1] - Pb[1] * M[k][0];
              J[k][3] = M[k][0];
              J[k][4] = M[k][1];
              J[k][5] = M[k][2];
            }
            const R om0 = -((R)a.info[e] * ev[0]) * s, om1 = -((R)a.info[e] * ev[1]) * s;
            int q = 0;
#pragma unroll
            for (int i = 0; i < 6; ++i) {
#pragma unroll
              for (int j = i; j < 6; ++j) acc[q++].add((J[0][i] * w) * J[0][j] + (J[1][i] * w) * J[1][j]);
            }
#pragma unroll
            for (int i = 0; i < 6; ++i) acc[21 + i].add(J[0][i] * om0 + J[1][i] * om1);
            acc[27].add(rho);
          }
#pragma unroll
          for (int k = 0; k < 28; ++k) {
            const Acc<R> wv = warp_sum_acc(acc[k]);
            if (lane == 0) red.part[wid][k] = wv;
          }
          __syncthreads();
          if (tid < 28) {
            Acc<R> t = red.part[0][tid];
            for (int w = 1; w < T / 32; ++w) t.add(red.part[w][tid]);
            const double v = t.value();
            if (tid < 21) {
              int r0 = 0, rem = tid;
              while (rem >= 6 - r0) {
                rem -= 6 - r0;
                ++r0;
              }
              s_H[6 * r0 + r0 + rem] = v;
              s_H[6 * (r0 + rem) + r0] = v;
            } else if (tid < 27) {
              s_b[tid - 21] = v;
            } else {
              s_chi = v;
            }
          }
          __syncthreads();
          if (tid == 0 && it == 0) {
            double m = 0;
            for (int i = 0; i < 6; ++i) m = fmax(m, fabs(s_H[7 * i]));
            s_lambda = a.tau * m;
            s_ni = 2.0;
          }
          // trials
          for (int trial = 0; trial < a.max_trials; ++trial) {
            __syncthreads();
            if (tid == 0) {
              s_solve_ok = solve6(s_H, s_lambda, s_b, s_x) ? 1 : 0;
              se3_exp_left(s_x, s_qt, s_cand);
              pose_of(s_cand, s_pcand);
            }
            __syncthreads();
            double cost = 0.0;
            {
              Acc<R> c;
              c.zero();
              for (int e = e0 + tid; e < e1; e += T) {
                if (a.level[e]) continue;
                const auto& C = cam_of(a, a.cam[e], R(0));
                R Pb[3], Pc[3], ev[2];
                xform(s_pcand, C, a.Xw + 3 * (size_t)e, Pb, Pc);
                const R chi2 = chi2_of<R>(C, Pc, a.obs + 2 * (size_t)e, a.info[e], ev);
                const R dl = (R)a.delta[e];
                c.add((robust && dl > R(0)) ? huber_rho<R>(chi2, dl) : chi2);
              }
              const Acc<R> wv = warp_sum_acc(c);
              if (lane == 0) red.part[wid][0] = wv;
              __syncthreads();
              if (tid == 0) {
                Acc<R> t = red.part[0][0];
                for (int w = 1; w < T / 32; ++w) t.add(red.part[w][0]);
                cost = t.value();
              }
            }
            if (tid == 0) {
              // optimization_algorithm_levenberg.cpp:113-139
              double tempChi = s_solve_ok ? cost : DBL_MAX;
              double sc = 0.0;
              for (int k = 0; k < 6; ++k) sc += s_x[k] * (s_lambda * s_x[k] + s_b[k]);
              const double rho = (s_chi - tempChi) / (sc + 1e-3);
              bool brk = false;
              if (rho > 0 && isfinite(tempChi)) {
                const double q = 2 * rho - 1;
                double alpha = 1. - q * q * q;
                alpha = fmin(alpha, 2. / 3.);
                s_lambda *= fmax(1. / 3., alpha);
                s_ni = 2;
                s_chi = tempChi;
                for (int k = 0; k < 7; ++k) s_qt[k] = s_cand[k];
              } else {
                s_lambda *= s_ni;
                s_ni *= 2;
                if (!isfinite(s_lambda)) brk = true;
              }
              const int done_trials = trial + (brk ? 0 : 1);
              s_flag_more = (!brk && rho < 0 && done_trials < a.max_trials) ? 1 : 0;
              if (!s_flag_more && (done_trials == a.max_trials || rho == 0 || !isfinite(s_lambda))) s_stop = 1;
              pose_of(s_qt, s_pose);
            }
            __syncthreads();
            if (!s_flag_more) break;
          }
        }
        __syncthreads();
      }
      // ---- filter: chi2 >= thr -> level 1 (src/PoseEstimation.cpp:98-116)
      if (tid == 0) pose_of(s_qt, s_pose);
      __syncthreads();
      int bad = 0;
      for (int e = e0 + tid; e < e1; e += T) {
        if (a.level[e]) continue;
        const auto& C = cam_of(a, a.cam[e], R(0));
        R Pb[3], Pc[3], ev[2];
        xform(s_pose, C, a.Xw + 3 * (size_t)e, Pb, Pc);
        const R chi2 = chi2_of<R>(C, Pc, a.obs + 2 * (size_t)e, a.info[e], ev);
        if ((float)chi2 >= a.thr) {
          a.level[e] = 1;
          ++bad;
        }
      }
      for (int o = 16; o >= 1; o >>= 1) bad += __shfl_xor_sync(0xffffffffu, bad, o);
      if (lane == 0) s_red[wid] = bad;
      __syncthreads();
      nBad = 0;
      for (int w = 0; w < T / 32; ++w) nBad += (int)s_red[w];
      __syncthreads();
      if (nInitial - nBad < 10) break;
    }
    if (tid == 0) {
      a.inliers[p] = nInitial - nBad;
      if (nInitial - nBad >= 10)
        for (int k = 0; k < 7; ++k) a.qt[8 * (size_t)p + k] = s_qt[k];
    }
    __syncthreads();
  }
}

struct TuneKey {
  int precision, n, e_bucket;
  bool operator<(const TuneKey& o) const {
    return std::tie(precision, n, e_bucket) < std::tie(o.precision, o.n, o.e_bucket);
  }
};
struct TuneVal {
  int threads, ctas_per_sm;
};
std::map<TuneKey, TuneVal> g_tuned;
std::mutex g_tune_mutex;

template <typename R>
cudaError_t launch(const BatchArgs& a, int threads, int grid, cudaStream_t st) {
  switch (threads) {
    case 128:
      k_pose_batch<R, 128><<<grid, 128, 0, st>>>(a);
      break;
    case 512:
      k_pose_batch<R, 512><<<grid, 512, 0, st>>>(a);
      break;
    default:
      k_pose_batch<R, 256><<<grid, 256, 0, st>>>(a);
      break;
  }
  return cudaGetLastError();
}

void cam_dev(const float* K, const float* T, CamD& d, CamF& f) {
  // T_cam_body float 4x4 -> rotation (orthonormalised through the quaternion
  // of Converter::toSE3Quat) and translation
  const double R0[9] = {T[0], T[1], T[2], T[4], T[5], T[6], T[8], T[9], T[10]};
  double x, y, z, w;
  const double tr = R0[0] + R0[4] + R0[8];
  if (tr > 0) {
    double s = std::sqrt(tr + 1.0);
    w = 0.5 * s;
    s = 0.5 / s;
    x = (R0[7] - R0[5]) * s;
    y = (R0[2] - R0[6]) * s;
    z = (R0[3] - R0[1]) * s;
  } else {
    int i = 0;
    if (R0[4] > R0[0]) i = 1;
    if (R0[8] > R0[4 * i]) i = 2;
    const int j = (i + 1) % 3, k = (j + 1) % 3;
    double s = std::sqrt(R0[4 * i] - R0[4 * j] - R0[4 * k] + 1.0);
    double v[3];
    v[i] = 0.5 * s;
    s = 0.5 / s;
    w = (R0[3 * k + j] - R0[3 * j + k]) * s;
    v[j] = (R0[3 * j + i] + R0[3 * i + j]) * s;
    v[k] = (R0[3 * k + i] + R0[3 * i + k]) * s;
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
  const double n = std::sqrt(x * x + y * y + z * z + w * w);
  x /= n;
  y /= n;
  z /= n;
  w /= n;
  const double tx = 2 * x, ty = 2 * y, tz = 2 * z;
  const double Rm[9] = {1 - (ty * y + tz * z), ty * x - tz * w, tz * x + ty * w,
                        ty * x + tz * w,       1 - (tx * x + tz * z), tz * y - tx * w,
                        tz * x - ty * w,       tz * y + tx * w,       1 - (tx * x + ty * y)};
  for (int k = 0; k < 4; ++k) {
    d.K[k] = K[k];
    f.K[k] = K[k];
  }
  d.bf = f.bf = 0;
  for (int k = 0; k < 9; ++k) {
    d.R[k] = Rm[k];
    f.R[k] = (float)Rm[k];
  }
  for (int k = 0; k < 3; ++k) {
    d.t[k] = T[4 * k + 3];
    f.t[k] = (float)T[4 * k + 3];
  }
}

}  // namespace
}  // namespace mcba

using namespace mcba;

extern "C" int mcba_batch_pose_only(int32_t device, int32_t precision, int32_t n, const int32_t* edge_begin,
                                    int32_t n_cams, const float* cam_K, const float* cam_Tcb,
                                    const int32_t* edge_cam, const float* edge_obs, const float* edge_Xw,
                                    const float* edge_info, const float* edge_delta, int32_t rounds,
                                    int32_t iterations, float chi2_threshold, int32_t drop_robust_round,
                                    double* poses_qt, uint8_t* edge_level, int32_t* inliers, double* ms_device) {
  if (n < 0 || !edge_begin || n_cams <= 0 || !cam_K || !cam_Tcb || !poses_qt || !inliers) return MCBA_ERR_INVALID;
  if (precision != MCBA_PREC_FP64 && precision != MCBA_PREC_MIXED) return MCBA_ERR_INVALID;
  if (n == 0) return MCBA_OK;
  const int E = edge_begin[n];
  if (edge_begin[0] != 0 || E < 0) return MCBA_ERR_INVALID;
  for (int i = 0; i < n; ++i)
    if (edge_begin[i + 1] < edge_begin[i]) return MCBA_ERR_INVALID;
  if (E > 0 && (!edge_cam || !edge_obs || !edge_Xw || !edge_info || !edge_delta || !edge_level))
    return MCBA_ERR_INVALID;
  for (int e = 0; e < E; ++e)
    if (edge_cam[e] < 0 || edge_cam[e] >= n_cams) return MCBA_ERR_INVALID;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return MCBA_ERR_NO_DEVICE;
  if (device < 0 || device >= ndev || cudaSetDevice(device) != cudaSuccess) return MCBA_ERR_NO_DEVICE;

  std::vector<CamD> cd(n_cams);
  std::vector<CamF> cf(n_cams);
  for (int c = 0; c < n_cams; ++c) cam_dev(cam_K + 4 * c, cam_Tcb + 16 * c, cd[c], cf[c]);
  std::vector<double> q8(8 * (size_t)n, 0.0);
  for (int i = 0; i < n; ++i) {
    double x = poses_qt[7 * i], y = poses_qt[7 * i + 1], z = poses_qt[7 * i + 2], w = poses_qt[7 * i + 3];
    if (w < 0) {
      x = -x;
      y = -y;
      z = -z;
      w = -w;
    }
    const double nn = std::sqrt(x * x + y * y + z * z + w * w);
    if (!(nn > 0)) return MCBA_ERR_INVALID;
    q8[8 * i] = x / nn;
    q8[8 * i + 1] = y / nn;
    q8[8 * i + 2] = z / nn;
    q8[8 * i + 3] = w / nn;
    for (int k = 0; k < 3; ++k) q8[8 * i + 4 + k] = poses_qt[7 * i + 4 + k];
  }

  // device buffers (owned by this call)
  void* buf = nullptr;
  const size_t sz_eb = sizeof(int) * (n + 1), sz_cam = sizeof(int) * E, sz_obs = sizeof(float) * 2 * (size_t)E,
               sz_X = sizeof(float) * 3 * (size_t)E, sz_f = sizeof(float) * (size_t)E,
               sz_cd = sizeof(CamD) * n_cams, sz_cf = sizeof(CamF) * n_cams, sz_q = sizeof(double) * 8 * (size_t)n,
               sz_lv = (size_t)E, sz_in = sizeof(int) * n;
  auto al = [](size_t s) { return (s + 255) & ~size_t(255); };
  const size_t total = al(sz_eb) + al(sz_cam) + al(sz_obs) + al(sz_X) + 2 * al(sz_f) + al(sz_cd) + al(sz_cf) +
                       2 * al(sz_q) + al(sz_lv) + al(sz_in) + 256;
  if (cudaMalloc(&buf, total) != cudaSuccess) return MCBA_ERR_NOMEM;
  char* pb = (char*)buf;
  auto take = [&](size_t s) {
    char* r = pb;
    pb += al(s);
    return r;
  };
  BatchArgs a{};
  a.n = n;
  int* d_eb = (int*)take(sz_eb);
  int* d_cam = (int*)take(sz_cam);
  float* d_obs = (float*)take(sz_obs);
  float* d_X = (float*)take(sz_X);
  float* d_info = (float*)take(sz_f);
  float* d_delta = (float*)take(sz_f);
  CamD* d_cd = (CamD*)take(sz_cd);
  CamF* d_cf = (CamF*)take(sz_cf);
  double* d_q = (double*)take(sz_q);
  double* d_q0 = (double*)take(sz_q);
  uint8_t* d_lv = (uint8_t*)take(sz_lv);
  int* d_in = (int*)take(sz_in);
  int* d_queue = (int*)take(256);
  cudaStream_t st;
  cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  int rc = MCBA_OK;
  auto ck = [&](cudaError_t e) {
    if (e != cudaSuccess && rc == MCBA_OK) rc = MCBA_ERR_CUDA;
  };
  ck(cudaMemcpyAsync(d_eb, edge_begin, sz_eb, cudaMemcpyHostToDevice, st));
  if (E) {
    ck(cudaMemcpyAsync(d_cam, edge_cam, sz_cam, cudaMemcpyHostToDevice, st));
    ck(cudaMemcpyAsync(d_obs, edge_obs, sz_obs, cudaMemcpyHostToDevice, st));
    ck(cudaMemcpyAsync(d_X, edge_Xw, sz_X, cudaMemcpyHostToDevice, st));
    ck(cudaMemcpyAsync(d_info, edge_info, sz_f, cudaMemcpyHostToDevice, st));
    ck(cudaMemcpyAsync(d_delta, edge_delta, sz_f, cudaMemcpyHostToDevice, st));
  }
  ck(cudaMemcpyAsync(d_cd, cd.data(), sz_cd, cudaMemcpyHostToDevice, st));
  ck(cudaMemcpyAsync(d_cf, cf.data(), sz_cf, cudaMemcpyHostToDevice, st));
  ck(cudaMemcpyAsync(d_q0, q8.data(), sz_q, cudaMemcpyHostToDevice, st));
  a.edge_begin = d_eb;
  a.cam = d_cam;
  a.obs = d_obs;
  a.Xw = d_X;
  a.info = d_info;
  a.delta = d_delta;
  a.cd = d_cd;
  a.cf = d_cf;
  a.qt = d_q;
  a.level = d_lv;
  a.inliers = d_in;
  a.queue = d_queue;
  a.rounds = rounds;
  a.iters = iterations;
  a.drop_round = drop_robust_round;
  a.max_trials = 10;
  a.thr = chi2_threshold;
  a.tau = 1e-5;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);

  // one run = reset the queue and the poses, persistent kernel; captured once
  // per configuration as a CUDA graph
  auto run = [&](int threads, int per_sm, float* ms) -> int {
    const int grid = std::max(1, std::min(n, sms * per_sm));
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    ck(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    ck(cudaMemsetAsync(d_queue, 0, sizeof(int), st));
    ck(cudaMemcpyAsync(d_q, d_q0, sz_q, cudaMemcpyDeviceToDevice, st));
    ck(precision == MCBA_PREC_MIXED ? launch<float>(a, threads, grid, st) : launch<double>(a, threads, grid, st));
    ck(cudaStreamEndCapture(st, &g));
    if (rc) return rc;
    ck(cudaGraphInstantiate(&ge, g, 0));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    ck(cudaEventRecord(e0, st));
    ck(cudaGraphLaunch(ge, st));
    ck(cudaEventRecord(e1, st));
    ck(cudaStreamSynchronize(st));
    if (ms) cudaEventElapsedTime(ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaGraphExecDestroy(ge);
    cudaGraphDestroy(g);
    return rc;
  };

  // autotune threads per CTA and CTAs per SM once per (precision, batch shape)
  TuneKey key{precision, n, 31 - __builtin_clz((unsigned)std::max(E, 1))};
  TuneVal best{256, 1};
  bool have = false;
  {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    auto it = g_tuned.find(key);
    if (it != g_tuned.end()) {
      best = it->second;
      have = true;
    }
  }
  if (!have) {
    float best_ms = 1e30f;
    for (int threads : {128, 256, 512})
      for (int per_sm : {1, 2}) {
        float ms = 0.f;
        if (run(threads, per_sm, &ms) != MCBA_OK) break;
        if (ms < best_ms) {
          best_ms = ms;
          best = {threads, per_sm};
        }
      }
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_tuned[key] = best;
  }
  float ms = 0.f;
  if (rc == MCBA_OK) run(best.threads, best.ctas_per_sm, &ms);
  if (ms_device) *ms_device = ms;
  if (rc == MCBA_OK) {
    std::vector<double> out(8 * (size_t)n);
    ck(cudaMemcpy(out.data(), d_q, sz_q, cudaMemcpyDeviceToHost));
    if (E && edge_level) ck(cudaMemcpy(edge_level, d_lv, sz_lv, cudaMemcpyDeviceToHost));
    ck(cudaMemcpy(inliers, d_in, sz_in, cudaMemcpyDeviceToHost));
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < 7; ++k) poses_qt[7 * i + k] = out[8 * i + k];
  }
  cudaStreamDestroy(st);
  cudaFree(buf);
  return rc;
}
