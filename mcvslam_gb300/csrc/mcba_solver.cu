// mcba_solver.cu -- GB300 Levenberg-Marquardt bundle-adjustment solver.
//
// One LM solve of MCVSLAM's BAoptimizer (g2o OptimizationAlgorithmLevenberg
// over BlockSolver<6,3> with Schur elimination of the points) as device
// kernels:
//   linearize      per-edge residual, Huber weight, Jacobians and quadratic
//                  form terms (base_binary_edge.hpp:64-136); pose terms
//                  reduced per CTA (one pose per CTA), point terms and Hpl
//                  written per edge in point-sorted order
//   pose/point reduce  deterministic segmented sums into Hpp, Hll, b
//   schur_edge     per edge Y = Hpl Dinv and q = Hpl Dinv b_l
//                  (block_solver.hpp:346-374)
//   schur_pairs    reduced camera blocks S_ab -= sum Y_i Hpl_j^T over the
//                  edge pairs of every block (block_solver.hpp:376-391),
//                  one warp per pair chunk, no atomics
//   chol_*         blocked FP64 Cholesky of the reduced camera system with
//                  b_schur as an extra row (forward substitution for free)
//   backsolve / backsub / update   x_p, x_l = Dinv(b_l - Hpl^T x_p), the SE3
//                  exp retraction and the point update, both into the other
//                  half of a double-buffered state (push/pop become a flip)
//   cost / decide  activeRobustChi2 and g2o's accept/reject, lambda and nu
//                  update (optimization_algorithm_levenberg.cpp:92-141) on
//                  the device.
// The linearisation real type R is double (plain) or float (mixed); the
// Cholesky, damping, gain ratio and retraction are FP64 in both.

#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstring>
#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "mcba_chol.h"
#include "mcba_chol_dev.cuh"
#include "mcba_chol_tiled.h"
#include "mcba_device.cuh"
#include "mcba_internal.h"

namespace mcba {
using namespace dev;

namespace {

// Per canonical edge row: Hpl 6x3 | Hll upper 6 | b_l 3 | pad = 28 reals.  FP32
// rows append the low halves of the float-float Hll terms (28..33) and pad
// to 36 floats (144 B, a multiple of 16 B).
template <typename R>
__host__ __device__ constexpr int row_stride() {
  return sizeof(R) == sizeof(double) ? 28 : 36;
}
constexpr int kHllLo = 28;
constexpr int kPdv = 12;   // per free point: (Hll + lambda I)^-1 row-major 9 | Dinv b_l 3
constexpr int kYQ = 24;    // per canonical edge: Y 6x3 | q 6
constexpr int kNB = 32;    // Cholesky tile
constexpr int kLinThreads = 256;
constexpr int kClusterCholMaxLd = 512;  // reduced systems up to 85 free keyframes use the cluster solve

// upper-triangle slot of a 6x6 entry (i <= j)
__host__ __device__ constexpr int u6(int i, int j) { return i * 6 - (i * (i - 1)) / 2 + (j - i); }
__host__ __device__ constexpr int u3(int i, int j) { return i * 3 - (i * (i - 1)) / 2 + (j - i); }

struct LMState {
  double lambda, ni, current_chi, temp_chi, rho, scale, initial_chi;
  int iteration, trial, cur, solve_ok;
  int trial_continue, terminate, total_trials, n_log;
  int max_trials, max_log, last_accepted, max_iters;
  int outer_runs, pad0;
  unsigned long long lam_bits;  // max |H_jj| as ordered IEEE bits (lambda init)
};

struct Bufs {
  // state (ping-pong)
  double* pose_qt[2];  // [K][8]
  PoseLinD* pd[2];
  PoseLinF* pf[2];
  double* Xd[2];       // [P+U][3]
  float4* Xf[2];
  CamD* cd;
  CamF* cf;
  // structure
  EdgeRec* recs;
  float* obs;
  int* chunk_begin;
  int* chunk_pose;
  int* pose_chunk_begin;
  int* pt_begin;
  int* canon_pose_h;
  int* canon_point_h;
  int2* pairs;
  int* pchunk_begin;
  int* block_ab;
  int* block_chunk_begin;
  int* pose_canon_begin;
  int* pose_canon_list;
  int* free_pose_ids;
  int* free_point_ids;
  // numeric workspaces (R-typed, stored as bytes)
  void* rows;       // [Ec][row_stride<R>()]
  void* partials;   // [nchunk][32] accumulators
  double* Hpp;      // [Kf][36] FP64 (formed from the accumulators)
  double* Hll;      // [Lf][6] FP64 (upper triangle of the point blocks)
  double* bp;       // [6Kf] FP64
  void* bl;         // [3Lf]
  void* pdv;        // [Lf][kPdv] damped point-block inverses of the current trial
  void* yq;         // [Ec][kYQ]
  void* ppart;      // [npchunk][36] accumulators
  void* qpart;      // [nchunk][6] accumulators of Hpl Dinv b_l per pose chunk
  double* S;        // [(ld+32) x ld]
  double* cws;      // workspace of the cluster or tiled factorisation
  double* dinv;     // [ld] reciprocal Cholesky diagonal
  double* x;        // [6Kf + 3Lf]
  double* cost_part;
  double* scale_part;
  int* done;  // [2] CTAs finished in k_cost_step / k_reduce (0 between launches)
  LMState* lm;
  mcba_trial_log* log;
};

template <typename R>
struct Ptrs {
  __host__ __device__ static R* p(void* v) { return reinterpret_cast<R*>(v); }
};

__device__ __forceinline__ StateView make_view(const Bufs& B, int which) {
  StateView v;
  v.pd = B.pd[which];
  v.pf = B.pf[which];
  v.Xd = B.Xd[which];
  v.Xf = B.Xf[which];
  v.cd = B.cd;
  v.cf = B.cf;
  return v;
}

// 16-byte vector access to per-edge rows (row strides are multiples of 16 B).
template <typename R, int N>
__device__ __forceinline__ void load_row(const R* p, R* v);
template <typename R, int N>
__device__ __forceinline__ void store_row(R* p, const R* v);
template <>
__device__ __forceinline__ void load_row<float, 20>(const float* p, float* v) {
  const float4* q = reinterpret_cast<const float4*>(p);
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    const float4 t = q[i];
    v[4 * i] = t.x;
    v[4 * i + 1] = t.y;
    v[4 * i + 2] = t.z;
    v[4 * i + 3] = t.w;
  }
}
template <>
__device__ __forceinline__ void load_row<double, 20>(const double* p, double* v) {
  const double2* q = reinterpret_cast<const double2*>(p);
#pragma unroll
  for (int i = 0; i < 10; ++i) {
    const double2 t = q[i];
    v[2 * i] = t.x;
    v[2 * i + 1] = t.y;
  }
}
template <>
__device__ __forceinline__ void load_row<double, 10>(const double* p, double* v) {
  const double2* q = reinterpret_cast<const double2*>(p);
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    const double2 t = q[i];
    v[2 * i] = t.x;
    v[2 * i + 1] = t.y;
  }
}
template <>
__device__ __forceinline__ void store_row<float, 20>(float* p, const float* v) {
  float4* q = reinterpret_cast<float4*>(p);
#pragma unroll
  for (int i = 0; i < 5; ++i) q[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
}
template <>
__device__ __forceinline__ void store_row<double, 20>(double* p, const double* v) {
  double2* q = reinterpret_cast<double2*>(p);
#pragma unroll
  for (int i = 0; i < 10; ++i) q[i] = make_double2(v[2 * i], v[2 * i + 1]);
}
template <>
__device__ __forceinline__ void store_row<float, 36>(float* p, const float* v) {
  float4* q = reinterpret_cast<float4*>(p);
#pragma unroll
  for (int i = 0; i < 9; ++i) q[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
}
template <>
__device__ __forceinline__ void store_row<float, 12>(float* p, const float* v) {
  float4* q = reinterpret_cast<float4*>(p);
#pragma unroll
  for (int i = 0; i < 3; ++i) q[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
}
template <>
__device__ __forceinline__ void store_row<double, 12>(double* p, const double* v) {
  double2* q = reinterpret_cast<double2*>(p);
#pragma unroll
  for (int i = 0; i < 6; ++i) q[i] = make_double2(v[2 * i], v[2 * i + 1]);
}
template <>
__device__ __forceinline__ void load_row<float, 12>(const float* p, float* v) {
  const float4* q = reinterpret_cast<const float4*>(p);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float4 t = q[i];
    v[4 * i] = t.x;
    v[4 * i + 1] = t.y;
    v[4 * i + 2] = t.z;
    v[4 * i + 3] = t.w;
  }
}
template <>
__device__ __forceinline__ void load_row<double, 12>(const double* p, double* v) {
  const double2* q = reinterpret_cast<const double2*>(p);
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    const double2 t = q[i];
    v[2 * i] = t.x;
    v[2 * i + 1] = t.y;
  }
}

// w * sum_k Jl[k][i] Jl[k][q] over the residual rows: one entry of an edge's
// point block.  FP64 rows evaluate it directly.  FP32 rows carry it as an
// unevaluated float-float pair (hi + lo): every product is split exactly by an
// FMA (TwoProduct) and the terms are added with TwoSum, all on FP32 pipes.
// The block of a point seen along nearly parallel rays is ill-conditioned, and
// its inverse enlarges the rounding of single FP32 entries by the condition
// number; the pair keeps those bits until the FP64 per-point sum.
template <typename R>
__device__ __forceinline__ void hll_entry(const R (&Jl)[3][3], R w, bool d3, int i, int q, R& hi, R& lo);
template <>
__device__ __forceinline__ void hll_entry<double>(const double (&Jl)[3][3], double w, bool d3, int i, int q,
                                                  double& hi, double& lo) {
  double h = (Jl[0][i] * w) * Jl[0][q] + (Jl[1][i] * w) * Jl[1][q];
  if (d3) h += (Jl[2][i] * w) * Jl[2][q];
  hi = h;
  lo = 0.0;
}
template <>
__device__ __forceinline__ void hll_entry<float>(const float (&Jl)[3][3], float w, bool d3, int i, int q, float& hi,
                                                 float& lo) {
  Acc<float> a;
  a.zero();
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (k == 2 && !d3) break;
    const float ah = __fmul_rn(Jl[k][i], w);
    const float al = __fmaf_rn(Jl[k][i], w, -ah);       // Jl_i w = ah + al exactly
    const float ph = __fmul_rn(ah, Jl[k][q]);
    const float pl = __fadd_rn(__fmaf_rn(ah, Jl[k][q], -ph), __fmul_rn(al, Jl[k][q]));
    a.add(ph);
    a.lo = __fadd_rn(a.lo, pl);
  }
  hi = __fadd_rn(a.hi, a.lo);
  lo = __fsub_rn(a.lo, __fsub_rn(hi, a.hi));
}
template <>
__device__ __forceinline__ void store_row<double, 28>(double* p, const double* v) {
  double2* q = reinterpret_cast<double2*>(p);
#pragma unroll
  for (int i = 0; i < 14; ++i) q[i] = make_double2(v[2 * i], v[2 * i + 1]);
}

// ------------------------------------------------------------ kernels --
// The kernels' bodies run on a "block": the CTA of a plain launch, or a
// group of warps of the persistent window kernel (k_windows), which runs
// the same bodies for virtual block ids it is dealt.  id / tid / nthr
// replace blockIdx.x / threadIdx.x / blockDim.x; sync() is __syncthreads for
// a whole CTA and a named barrier of the block's warps otherwise.
struct Blk {
  int id, tid, nthr, bar;
  __device__ __forceinline__ void sync() const {
    if (bar == 0)
      __syncthreads();
    else
      asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(nthr) : "memory");
  }
};
__device__ __forceinline__ Blk grid_blk() { return Blk{(int)blockIdx.x, (int)threadIdx.x, (int)blockDim.x, 0}; }

// The kernels of the LM chain are launched with programmatic stream
// serialisation: a kernel's launch overlaps the end of the one before it,
// and its first instruction waits until that grid has completed and its
// writes are visible (a no-op for a plain launch).
__device__ __forceinline__ void chain_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// block_sum over a Blk (same tree as dev::block_sum for the same block size)
template <typename T>
__device__ __forceinline__ T blk_sum(T x, T* sh, const Blk& b) {
  const int lane = b.tid & 31, wid = b.tid >> 5, nw = b.nthr >> 5;
  x = warp_sum(x);
  b.sync();
  if (lane == 0) sh[wid] = x;
  b.sync();
  T r = (lane < nw) ? sh[lane] : T(0);
  r = warp_sum(r);
  return r;
}

// Start of one LM iteration (the trial loop's state).
__device__ __forceinline__ void iter_begin(LMState* lm) {
  lm->trial = 0;
  lm->trial_continue = 1;
}

__device__ __forceinline__ void pose_lin_one(const double* q, PoseLinD* pd, PoseLinF* pf) {
  double Rm[9];
  quat_to_R(q, Rm);
  PoseLinD d;
  PoseLinF f;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    d.R[k] = Rm[k];
    f.R[k] = (float)Rm[k];
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) d.t[k] = q[4 + k];
#pragma unroll
  for (int k = 0; k < 3; ++k)
    f.c[k] = (float)(-(Rm[k] * q[4] + Rm[3 + k] * q[5] + Rm[6 + k] * q[6]));
  *pd = d;
  *pf = f;
}

// Both halves of the double-buffered state, with their rotation matrices
// and float copies, from one source (the uploaded state or the saved
// initial one), in one launch; keep_q / keep_x (may be null) also receive
// the source, as the saved initial state.
struct SpreadArgs {
  const double* src_q;
  const double* src_x;
  int K, NP;
  double* q[2];
  double* x[2];
  PoseLinD* pd[2];
  PoseLinF* pf[2];
  float4* xf[2];
  double* keep_q;
  double* keep_x;
};

__global__ void k_spread(SpreadArgs a) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.K + a.NP; i += gridDim.x * blockDim.x) {
    if (i < a.K) {
      double q[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) q[k] = a.src_q[8 * (size_t)i + k];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        a.q[0][8 * (size_t)i + k] = q[k];
        a.q[1][8 * (size_t)i + k] = q[k];
        if (a.keep_q) a.keep_q[8 * (size_t)i + k] = q[k];
      }
      pose_lin_one(q, a.pd[0] + i, a.pf[0] + i);
      a.pd[1][i] = a.pd[0][i];
      a.pf[1][i] = a.pf[0][i];
    } else {
      const size_t j = (size_t)(i - a.K);
      const double x0 = a.src_x[3 * j], x1 = a.src_x[3 * j + 1], x2 = a.src_x[3 * j + 2];
      const float4 f = make_float4((float)x0, (float)x1, (float)x2, 0.f);
#pragma unroll
      for (int b = 0; b < 2; ++b) {
        a.x[b][3 * j] = x0;
        a.x[b][3 * j + 1] = x1;
        a.x[b][3 * j + 2] = x2;
        a.xf[b][j] = f;
      }
      if (a.keep_x) {
        a.keep_x[3 * j] = x0;
        a.keep_x[3 * j + 1] = x1;
        a.keep_x[3 * j + 2] = x2;
      }
    }
  }
}

// Per-edge linearisation (buildSystem's edge loop, block_solver.hpp:490-506).
template <typename R>
__device__ __forceinline__ void linearize_blk(const Bufs& B, const Blk& b, Acc<R> (*sh)[32]) {
  const int c = b.id;
  const int jb = B.chunk_begin[c], je = B.chunk_begin[c + 1];
  const int ph = B.chunk_pose[c];
  const int j = jb + b.tid;
  const StateView v = make_view(B, B.lm->cur);
  Acc<R> acc[32];
#pragma unroll
  for (int k = 0; k < 32; ++k) acc[k].zero();
  if (j < je) {
    const EdgeRec r = B.recs[j];
    const float obs[3] = {B.obs[3 * (size_t)j], B.obs[3 * (size_t)j + 1], B.obs[3 * (size_t)j + 2]};
    R Pb[3], Pc[3], e[3], chi2;
    transform(r, v, Pb, Pc);
    edge_error<R>(r, obs, v, Pc, e, chi2);
    const R info = (R)r.info;
    R s = R(1);
    if (r.robust) s = huber_d1<R>(chi2, (R)r.delta);
    const R w = s * info;
    R Jl[3][3], Jp[3][6];
    edge_jac<R>(r, v, Pb, Pc, Jl, Jp);
    R om[3];
    const bool d3 = r.dim == 3;
#pragma unroll
    for (int k = 0; k < 3; ++k) om[k] = (k < 2 || d3) ? -(info * e[k]) * s : R(0);
    R wJp[3][6];
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int i = 0; i < 6; ++i) wJp[k][i] = (k < 2 || d3) ? Jp[k][i] * w : R(0);
    if (r.point_h >= 0) {
      R* row = Ptrs<R>::p(B.rows) + (size_t)r.canon * row_stride<R>();
      R out[row_stride<R>()];
#pragma unroll
      for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          R h = R(0);
          if (r.pose_h >= 0) {
            h = wJp[0][i] * Jl[0][q] + wJp[1][i] * Jl[1][q];
            if (d3) h += wJp[2][i] * Jl[2][q];
          }
          out[i * 3 + q] = h;
        }
#pragma unroll
      for (int i = 0; i < 3; ++i) {
#pragma unroll
        for (int q = i; q < 3; ++q) {
          R lo;
          hll_entry<R>(Jl, w, d3, i, q, out[18 + u3(i, q)], lo);
          if constexpr (row_stride<R>() > kHllLo) out[kHllLo + u3(i, q)] = lo;
        }
        R bb = Jl[0][i] * om[0] + Jl[1][i] * om[1];
        if (d3) bb += Jl[2][i] * om[2];
        out[24 + i] = bb;
      }
      out[27] = R(0);
#pragma unroll
      for (int k = kHllLo + 6; k < row_stride<R>(); ++k) out[k] = R(0);
      store_row<R, row_stride<R>()>(row, out);
    }
    if (r.pose_h >= 0) {
#pragma unroll
      for (int i = 0; i < 6; ++i) {
#pragma unroll
        for (int q = i; q < 6; ++q) {
          R h = wJp[0][i] * Jp[0][q] + wJp[1][i] * Jp[1][q];
          if (d3) h += wJp[2][i] * Jp[2][q];
          acc[u6(i, q)].add(h);
        }
        R bb = Jp[0][i] * om[0] + Jp[1][i] * om[1];
        if (d3) bb += Jp[2][i] * om[2];
        acc[21 + i].add(bb);
      }
    }
  }
  if (ph >= 0) {
    const Acc<R> mine = warp_reduce_scatter32_acc(acc);
    sh[b.tid >> 5][b.tid & 31] = mine;
    b.sync();
    if (b.tid < 32) {
      Acc<R> t = sh[0][b.tid];
#pragma unroll
      for (int w = 1; w < kLinThreads / 32; ++w) t.add(sh[w][b.tid]);
      reinterpret_cast<Acc<R>*>(B.partials)[(size_t)c * 32 + b.tid] = t;
    }
  }
}

// The first kernel of an LM iteration: its first thread also starts the
// iteration (trial count, trial loop armed; in a graph it re-arms the trial
// loop's condition, whose default applies only when the whole graph is
// launched).
template <typename R>
__global__ void __launch_bounds__(kLinThreads) k_linearize(Bufs B, cudaGraphConditionalHandle h_trial, int in_graph) {
  __shared__ Acc<R> sh[kLinThreads / 32][32];
  chain_wait();
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    iter_begin(B.lm);
    if (in_graph) cudaGraphSetConditional(h_trial, 1u);
  }
  linearize_blk<R>(B, grid_blk(), sh);
}

// a += p[c0 * stride] + .. + p[(c1 - 1) * stride], in that order; the loads
// go out eight at a time, so a long range costs a few L2 round trips, not
// one per term.
template <typename R>
__device__ __forceinline__ void acc_range(Acc<R>& a, const Acc<R>* p, int c0, int c1, size_t stride) {
  int c = c0;
  for (; c + 8 <= c1; c += 8) {
    Acc<R> v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = p[(size_t)(c + u) * stride];
#pragma unroll
    for (int u = 0; u < 8; ++u) a.add(v[u]);
  }
  for (; c < c1; ++c) a.add(p[(size_t)c * stride]);
}

// Hpp / b_p: sum of the chunk partials of each free pose (warp per pose),
// stored in FP64.
template <typename R>
__device__ __forceinline__ void pose_reduce_warp(const Bufs& B, int Kf, int i, int lane) {
  if (i >= Kf) return;
  const int c0 = B.pose_chunk_begin[i], c1 = B.pose_chunk_begin[i + 1];
  const Acc<R>* part = reinterpret_cast<const Acc<R>*>(B.partials);
  Acc<R> a;
  a.zero();
  acc_range(a, part + lane, c0, c1, 32);
  const double s = a.value();
  double* H = B.Hpp + (size_t)i * 36;
  if (lane < 21) {
    int r = 0, rem = lane;
    while (rem >= 6 - r) {
      rem -= 6 - r;
      ++r;
    }
    const int bcol = r + rem;
    H[r * 6 + bcol] = s;
    H[bcol * 6 + r] = s;
  } else if (lane < 27) {
    B.bp[6 * (size_t)i + (lane - 21)] = s;
  }
}

// Hll / b_l: sum over the (<= a few) edges of each free point.
// Hll is stored in FP64: FP32 rows sum their float-float pairs with TwoSum
// (Acc<float>: the high parts exactly, the low parts and the TwoSum errors in
// a second float) and convert once per point; b_l stays in the linearisation
// type.
template <typename R>
__device__ __forceinline__ void point_reduce_thread(const Bufs& B, int Lf, int l) {
  if (l >= Lf) return;
  const int e0 = B.pt_begin[l], e1 = B.pt_begin[l + 1];
  Acc<R> h[6];
  R s[3];
#pragma unroll
  for (int k = 0; k < 6; ++k) h[k].zero();
#pragma unroll
  for (int k = 0; k < 3; ++k) s[k] = R(0);
#pragma unroll 4
  for (int e = e0; e < e1; ++e) {
    const R* row = Ptrs<R>::p(B.rows) + (size_t)e * row_stride<R>();
    // the row's Hll, b_l (and low halves) by 16-byte loads: entries 16..35
    // of an FP32 row, 18..27 of an FP64 row
    R hv[6], bv[3], lov[6];
    if constexpr (row_stride<R>() > kHllLo) {
      R t[20];
      load_row<R, 20>(row + 16, t);
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        hv[k] = t[2 + k];
        lov[k] = t[kHllLo - 16 + k];
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) bv[k] = t[8 + k];
    } else {
      R t[10];
      load_row<R, 10>(row + 18, t);
#pragma unroll
      for (int k = 0; k < 6; ++k) hv[k] = t[k];
#pragma unroll
      for (int k = 0; k < 3; ++k) bv[k] = t[6 + k];
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      h[k].add(hv[k]);
      if constexpr (row_stride<R>() > kHllLo) h[k].lo = __fadd_rn(h[k].lo, lov[k]);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) s[k] += bv[k];
  }
  double* H = B.Hll + (size_t)l * 6;
#pragma unroll
  for (int k = 0; k < 6; ++k) H[k] = h[k].value();
  R* b = Ptrs<R>::p(B.bl) + 3 * (size_t)l;
#pragma unroll
  for (int k = 0; k < 3; ++k) b[k] = s[k];
}

// Both reductions in one launch of 128-thread blocks: the first blocks take
// four free poses each (a warp per pose), the rest 128 free points each.


// computeLambdaInit (optimization_algorithm_levenberg.cpp:145-157):
// tau * max |H_jj| over every free vertex (poses and points): a grid-wide
// maximum (atomicMax on the bit pattern) and then the scaling.
// |x| as an order-preserving integer: for non-negative doubles the IEEE bit
// pattern orders like the value, so the maximum needs no FP64 instruction.
__device__ __forceinline__ unsigned long long abs_bits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
}

// Thread `t` of `nt` takes entries t, t + nt, ..; the maximum does not
// depend on the split.
template <typename R>
__device__ __forceinline__ unsigned long long lambda_max_part(const Bufs& B, int Kf, int Lf, int t, int nt) {
  unsigned long long m = 0;
  const int n = 6 * Kf + 3 * Lf;
  for (int k = t; k < n; k += nt) {
    unsigned long long v;
    if (k < 6 * Kf) {
      v = abs_bits(B.Hpp[(size_t)(k / 6) * 36 + 7 * (k % 6)]);
    } else {
      const int i = k - 6 * Kf, d = i % 3;
      v = abs_bits(B.Hll[(size_t)(i / 3) * 6 + (d == 0 ? 0 : d == 1 ? 3 : 5)]);
    }
    m = v > m ? v : m;
  }
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    const unsigned long long v = __shfl_xor_sync(0xffffffffu, m, o);
    m = v > m ? v : m;
  }
  return m;
}


__device__ __forceinline__ void lambda_set(LMState* lm, double tau) {
  if (lm->iteration != 0) return;
  lm->lambda = tau * __longlong_as_double((long long)lm->lam_bits);
  lm->ni = 2.0;
}

// Both reductions in one launch of 128-thread blocks: the first blocks take
// four free poses each (a warp per pose), the rest 128 free points each.  In
// the first iteration the launch also forms computeLambdaInit's maximum
// (every block's maximum of its diagonal entries into lam_bits), and the
// last block to finish sets lambda from it.
template <typename R>
__global__ void k_reduce(Bufs B, int Kf, int Lf, int npose_blocks, double tau) {
  __shared__ int s_last;
  chain_wait();
  const int blk = blockIdx.x;
  const int lane = threadIdx.x & 31;
  int idx;
  if (blk < npose_blocks) {
    idx = 4 * blk + (threadIdx.x >> 5);
    pose_reduce_warp<R>(B, Kf, idx, lane);
  } else {
    idx = (blk - npose_blocks) * blockDim.x + threadIdx.x;
    point_reduce_thread<R>(B, Lf, idx);
  }
  if (B.lm->iteration != 0) return;
  // the diagonal entries this thread stored (Hpp's diagonal on the pose
  // warps' lanes 0, 6, 11, 15, 18, 20; Hll's three for a point's thread)
  unsigned long long m = 0;
  if (blk < npose_blocks) {
    if (idx < Kf && (lane == 0 || lane == 6 || lane == 11 || lane == 15 || lane == 18 || lane == 20)) {
      const int r = lane == 0 ? 0 : lane == 6 ? 1 : lane == 11 ? 2 : lane == 15 ? 3 : lane == 18 ? 4 : 5;
      m = abs_bits(B.Hpp[(size_t)idx * 36 + 7 * r]);
    }
  } else if (idx < Lf) {
    const double* H = B.Hll + (size_t)idx * 6;
    const unsigned long long a = abs_bits(H[0]), b = abs_bits(H[3]), c = abs_bits(H[5]);
    m = a > b ? a : b;
    m = c > m ? c : m;
  }
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    const unsigned long long v = __shfl_xor_sync(0xffffffffu, m, o);
    m = v > m ? v : m;
  }
  if (lane == 0 && m) atomicMax(&B.lm->lam_bits, m);
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(&B.done[1], 1) == (int)gridDim.x - 1;
  }
  __syncthreads();
  if (s_last && threadIdx.x == 0) {
    __threadfence();
    B.done[1] = 0;
    lambda_set(B.lm, tau);
  }
}

template <typename R>
__device__ __forceinline__ void damped_inverse(const R* Hu, R lam, R* Di) {
  const R d00 = Hu[0] + lam, d01 = Hu[1], d02 = Hu[2], d11 = Hu[3] + lam, d12 = Hu[4], d22 = Hu[5] + lam;
  const R c00 = d11 * d22 - d12 * d12;
  const R c01 = d12 * d02 - d01 * d22;
  const R c02 = d01 * d12 - d11 * d02;
  const R det = d00 * c00 + d01 * c01 + d02 * c02;
  const R id = R(1) / det;
  Di[0] = c00 * id;
  Di[1] = c01 * id;
  Di[2] = c02 * id;
  Di[3] = c01 * id;
  Di[4] = (d00 * d22 - d02 * d02) * id;
  Di[5] = (d02 * d01 - d00 * d12) * id;
  Di[6] = c02 * id;
  Di[7] = Di[5];
  Di[8] = (d00 * d11 - d01 * d01) * id;
}

// (Hll + lambda I)^-1 and Dinv b_l of every free point for the current trial
// (block_solver.hpp:346-354 inverts each landmark's damped block), in FP64
// from the FP64 point blocks, stored in the linearisation type:
// pdv[l] = Dinv row-major (9) | Dinv b_l (3).
template <typename R>
__device__ __forceinline__ void point_dinv_one(const Bufs& B, int l) {
  double D[9];
  damped_inverse<double>(B.Hll + (size_t)l * 6, B.lm->lambda, D);
  const R* bl = Ptrs<R>::p(B.bl) + 3 * (size_t)l;
  const double b0 = (double)bl[0], b1 = (double)bl[1], b2 = (double)bl[2];
  R o[kPdv];
#pragma unroll
  for (int k = 0; k < 9; ++k) o[k] = (R)D[k];
#pragma unroll
  for (int i = 0; i < 3; ++i) o[9 + i] = (R)(D[3 * i] * b0 + D[3 * i + 1] * b1 + D[3 * i + 2] * b2);
  store_row<R, kPdv>(Ptrs<R>::p(B.pdv) + (size_t)l * kPdv, o);
}

template <typename R>
__global__ void __launch_bounds__(128) k_point_dinv(Bufs B, int Lf) {
  chain_wait();
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l < Lf) point_dinv_one<R>(B, l);
}

// Y_e = Hpl_e Dinv for every edge with a free point and a free pose, walked in
// the pose-sorted stream (one pose per CTA) so that q = sum_e Hpl_e Dinv b_l
// -- the coefficient subtracted from b_p (block_solver.hpp:356-374) -- is
// reduced per chunk without atomics.
template <typename R>
__device__ __forceinline__ void schur_edge_blk(const Bufs& B, const Blk& b, Acc<R> (*sh)[kLinThreads / 32]) {
  const int c = b.id;
  const int jb = B.chunk_begin[c], je = B.chunk_begin[c + 1];
  const int ph = B.chunk_pose[c];
  const int j = jb + b.tid;
  Acc<R> qa[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) qa[k].zero();
  if (j < je) {
    const EdgeRec r = B.recs[j];
    if (r.canon >= 0 && r.pose_h >= 0) {
      const int e = r.canon, l = r.point_h;
      R Di[kPdv];
      load_row<R, kPdv>(Ptrs<R>::p(B.pdv) + (size_t)l * kPdv, Di);
      const R* db = Di + 9;
      R h[20];
      load_row<R, 20>(Ptrs<R>::p(B.rows) + (size_t)e * row_stride<R>(), h);
      R y[20];
#pragma unroll
      for (int rr = 0; rr < 6; ++rr) {
#pragma unroll
        for (int cc = 0; cc < 3; ++cc)
          y[rr * 3 + cc] = h[rr * 3] * Di[cc] + h[rr * 3 + 1] * Di[3 + cc] + h[rr * 3 + 2] * Di[6 + cc];
        qa[rr].add(h[rr * 3] * db[0] + h[rr * 3 + 1] * db[1] + h[rr * 3 + 2] * db[2]);
      }
      y[18] = R(0);
      y[19] = R(0);
      store_row<R, 20>(Ptrs<R>::p(B.yq) + (size_t)e * kYQ, y);
    }
  }
  if (ph >= 0) {
    const int lane = b.tid & 31, wid = b.tid >> 5;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const Acc<R> w = warp_sum_acc(qa[k]);
      if (lane == 0) sh[k][wid] = w;
    }
    b.sync();
    if (b.tid < 6) {
      Acc<R> t = sh[b.tid][0];
#pragma unroll
      for (int w = 1; w < kLinThreads / 32; ++w) t.add(sh[b.tid][w]);
      reinterpret_cast<Acc<R>*>(B.qpart)[(size_t)c * 6 + b.tid] = t;
    }
  }
}

template <typename R>
__global__ void __launch_bounds__(kLinThreads) k_schur_edge(Bufs B) {
  __shared__ Acc<R> sh[6][kLinThreads / 32];
  chain_wait();
  schur_edge_blk<R>(B, grid_blk(), sh);
}

// Reduced-camera block products over the pair list: one warp per chunk of
// <= 128 pairs that all belong to one block; lanes accumulate whole 6x6
// products in registers, then a reduce-scatter gives one partial per chunk.
template <typename R>
__device__ __forceinline__ void schur_pairs_warp(const Bufs& B, int warp, int lane) {
  const int p0 = B.pchunk_begin[warp], p1 = B.pchunk_begin[warp + 1];
  Acc<R> acc[32], acc2[4];
#pragma unroll
  for (int k = 0; k < 32; ++k) acc[k].zero();
#pragma unroll
  for (int k = 0; k < 4; ++k) acc2[k].zero();
  const R* yq = Ptrs<R>::p(B.yq);
  const R* rows = Ptrs<R>::p(B.rows);
  for (int p = p0 + lane; p < p1; p += 32) {
    const int2 ij = B.pairs[p];
    const R* Y = yq + (size_t)ij.x * kYQ;
    const R* H = rows + (size_t)ij.y * row_stride<R>();
    R y[20], h[20];
    load_row<R, 20>(Y, y);
    load_row<R, 20>(H, h);
#pragma unroll
    for (int r = 0; r < 6; ++r)
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        const R v = y[r * 3] * h[c * 3] + y[r * 3 + 1] * h[c * 3 + 1] + y[r * 3 + 2] * h[c * 3 + 2];
        const int t = r * 6 + c;
        if (t < 32)
          acc[t].add(v);
        else
          acc2[t - 32].add(v);
      }
  }
  const Acc<R> mine = warp_reduce_scatter32_acc(acc);
  Acc<R>* out = reinterpret_cast<Acc<R>*>(B.ppart) + (size_t)warp * 36;
  out[lane] = mine;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const Acc<R> s = warp_sum_acc(acc2[k]);
    if (lane == 0) out[32 + k] = s;
  }
}

template <typename R>
__global__ void __launch_bounds__(256) k_schur_pairs(Bufs B, int npc) {
  chain_wait();
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp < npc) schur_pairs_warp<R>(B, warp, threadIdx.x & 31);
}

// S_ab = [a == b](Hpp_a + lambda I) - sum of the block's chunk partials, into
// the dense FP64 reduced camera matrix (lower triangle is what the
// factorisation reads).  Four groups of 64 threads each sum a quarter of the
// block's chunks (36 entries per group), and the quarters meet in a fixed
// order, so a diagonal block's long run of chunks is four short dependent
// load chains.  For a diagonal block, group 1 forms b_schur meanwhile.
constexpr int kAsmGroups = 4;

template <typename R>
__device__ __forceinline__ void schur_assemble_blk(const Bufs& B, const Blk& b, int ld, Acc<R> (*sh)[36]) {
  const int blk = b.id;
  const int grp = b.tid >> 6, t = b.tid & 63;
  const int a = B.block_ab[2 * blk], bb = B.block_ab[2 * blk + 1];
  const int c0 = B.block_chunk_begin[blk], c1 = B.block_chunk_begin[blk + 1];
  if (t < 36) {
    const int len = c1 - c0;
    const int g0 = c0 + (int)(((long long)len * grp) / kAsmGroups);
    const int g1 = c0 + (int)(((long long)len * (grp + 1)) / kAsmGroups);
    const Acc<R>* part = reinterpret_cast<const Acc<R>*>(B.ppart);
    Acc<R> v;
    v.zero();
    acc_range(v, part + t, g0, g1, 36);
    sh[grp][t] = v;
  }
  if (a == bb && grp == 1 && t < 6) {
    // b_schur = b_p - sum of the pose's q chunk partials
    const Acc<R>* qp = reinterpret_cast<const Acc<R>*>(B.qpart);
    Acc<R> qs;
    qs.zero();
    acc_range(qs, qp + t, B.pose_chunk_begin[a], B.pose_chunk_begin[a + 1], 6);
    B.S[(size_t)ld * ld + 6 * a + t] = B.bp[6 * (size_t)a + t] - qs.value();
  }
  b.sync();
  if (grp != 0 || t >= 36) return;
  Acc<R> v = sh[0][t];
#pragma unroll
  for (int g = 1; g < kAsmGroups; ++g) v.add(sh[g][t]);
  const int r = t / 6, q = t % 6;
  if (a == bb) {
    double d = B.Hpp[(size_t)a * 36 + t] - v.value();
    if (r == q) d += B.lm->lambda;
    B.S[(size_t)(6 * a + r) * ld + 6 * a + q] = d;
  } else {
    const double d = -v.value();
    B.S[(size_t)(6 * a + r) * ld + 6 * bb + q] = d;
    B.S[(size_t)(6 * bb + q) * ld + 6 * a + r] = d;
  }
}

template <typename R>
__global__ void __launch_bounds__(64 * kAsmGroups) k_schur_assemble(Bufs B, int ld) {
  __shared__ Acc<R> sh[kAsmGroups][36];
  chain_wait();
  schur_assemble_blk<R>(B, grid_blk(), ld, sh);
}

// Landmark back-substitution (block_solver.hpp:420-446) and point update,
// plus the point part of computeScale (optimization_algorithm_levenberg.cpp:159-165).
// Four lanes per point: lane s of the group walks edges s, s+4, .. of the
// point (so the dependent index -> row/x loads of a point's edges are in
// flight together), the four partial sums meet in a fixed shuffle tree, and
// lanes 0-2 then update one coordinate each.
constexpr int kPtLanes = 4;
constexpr int kPtsPerBlock = 128 / kPtLanes;  // k_update runs 128-thread blocks

template <typename R>
__device__ __forceinline__ void backsub_block(const Bufs& B, int Lf, int n, int blk, double* sh, const Blk& b) {
  const int l = blk * kPtsPerBlock + b.tid / kPtLanes;
  const int sub = b.tid % kPtLanes;
  const int cur = B.lm->cur, cand = cur ^ 1;
  const double lam = B.lm->lambda;
  const bool ok = B.lm->solve_ok != 0;
  double sc = 0.0;
  R t[3] = {R(0), R(0), R(0)};
  if (l < Lf && ok) {
    const int e1 = B.pt_begin[l + 1];
#pragma unroll 2
    for (int e = B.pt_begin[l] + sub; e < e1; e += kPtLanes) {
      const int ph = B.canon_pose_h[e];
      if (ph < 0) continue;
      R H[20];
      load_row<R, 20>(Ptrs<R>::p(B.rows) + (size_t)e * row_stride<R>(), H);
      const double* xp = B.x + 6 * (size_t)ph;
      R xr[6];
#pragma unroll
      for (int k = 0; k < 6; ++k) xr[k] = (R)xp[k];
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        R u = R(0);
#pragma unroll
        for (int k = 0; k < 6; ++k) u += H[k * 3 + q] * xr[k];
        t[q] += u;
      }
    }
  }
  // the four lanes of a point are adjacent: partial sums meet as (0+1)+(2+3)
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    t[q] += __shfl_xor_sync(0xffffffffu, t[q], 1);
    t[q] += __shfl_xor_sync(0xffffffffu, t[q], 2);
  }
  if (l < Lf && sub < 3) {
    const int q = sub;
    const R* bl = Ptrs<R>::p(B.bl) + 3 * (size_t)l;
    double* xl = B.x + n + 3 * (size_t)l;
    if (ok) {
      const R cl[3] = {bl[0] - t[0], bl[1] - t[1], bl[2] - t[2]};
      const R* Dq = Ptrs<R>::p(B.pdv) + (size_t)l * kPdv + 3 * q;  // row q of Dinv
      xl[q] = (double)(Dq[0] * cl[0] + Dq[1] * cl[1] + Dq[2] * cl[2]);
    }
    const int id = B.free_point_ids[l];
    const double d = xl[q];
    const double nx = B.Xd[cur][3 * (size_t)id + q] + d;
    B.Xd[cand][3 * (size_t)id + q] = nx;
    sc = d * (lam * d + (double)bl[q]);
    reinterpret_cast<float*>(B.Xf[cand] + id)[q] = (float)nx;
    if (q == 0) reinterpret_cast<float*>(B.Xf[cand] + id)[3] = 0.f;
  }
  const double tot = blk_sum(sc, sh, b);
  if (b.tid == 0) B.scale_part[blk] = tot;
}

// VertexSE3Expmap::oplusImpl on every free pose into the candidate buffer,
// plus the pose part of computeScale.  Written to scale_part[slot].
template <typename R>
__device__ __forceinline__ void update_poses_block(const Bufs& B, int Kf, int slot0, int blk, double* sh,
                                                   const Blk& b) {
  const int i = blk * b.nthr + b.tid;
  const int cur = B.lm->cur, cand = cur ^ 1;
  const double lam = B.lm->lambda;
  double sc = 0.0;
  if (i < Kf) {
    const int id = B.free_pose_ids[i];
    const double* u = B.x + 6 * (size_t)i;
    double out[7];
    se3_exp_left(u, B.pose_qt[cur] + 8 * (size_t)id, out);
    double* dst = B.pose_qt[cand] + 8 * (size_t)id;
#pragma unroll
    for (int k = 0; k < 7; ++k) dst[k] = out[k];
    double Rm[9];
    quat_to_R(out, Rm);
    PoseLinD d;
    PoseLinF f;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      d.R[k] = Rm[k];
      f.R[k] = (float)Rm[k];
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      d.t[k] = out[4 + k];
      f.c[k] = (float)(-(Rm[k] * out[4] + Rm[3 + k] * out[5] + Rm[6 + k] * out[6]));
    }
    B.pd[cand][id] = d;
    B.pf[cand][id] = f;
#pragma unroll
    for (int k = 0; k < 6; ++k) sc += u[k] * (lam * u[k] + B.bp[6 * (size_t)i + k]);
  }
  const double tot = blk_sum(sc, sh, b);
  if (b.tid == 0) B.scale_part[slot0 + blk] = tot;
}

// One launch for both updates: the pose blocks (long FP64 exp chains) come
// first so that they start early and overlap the point blocks.  Scale
// partials keep their slots (points first, then poses), so the sum order
// does not depend on the launch layout.
template <typename R>
__device__ __forceinline__ void update_blk(const Bufs& B, const Blk& b, int Lf, int n, int Kf, int npose_blocks,
                                           int npt_blocks, double* sh) {
  if (b.id < npose_blocks)
    update_poses_block<R>(B, Kf, npt_blocks, b.id, sh, b);
  else
    backsub_block<R>(B, Lf, n, b.id - npose_blocks, sh, b);
}

template <typename R>
__global__ void k_update(Bufs B, int Lf, int n, int Kf, int npose_blocks, int npt_blocks) {
  __shared__ double sh[32];
  chain_wait();
  update_blk<R>(B, grid_blk(), Lf, n, Kf, npose_blocks, npt_blocks, sh);
}

// activeRobustChi2 (sparse_optimizer.cpp:102-116) at the current (which = 0)
// or candidate (which = 1) state: one partial per CTA.  FP32 edges are
// summed per warp as float-float pairs (TwoSum, ~48-bit significand), so
// the FP64 pipe, which is slow on this part, sees only the eight warp sums.
template <typename R>
__device__ __forceinline__ void cost_blk(const Bufs& B, const Blk& b, int E, int which, double* sh) {
  const int j = b.id * b.nthr + b.tid;
  const StateView v = make_view(B, B.lm->cur ^ which);
  R rho = R(0);
  if (j < E) {
    const EdgeRec r = B.recs[j];
    const float obs[3] = {B.obs[3 * (size_t)j], B.obs[3 * (size_t)j + 1], B.obs[3 * (size_t)j + 2]};
    R Pb[3], Pc[3], e[3], chi2;
    transform(r, v, Pb, Pc);
    edge_error<R>(r, obs, v, Pc, e, chi2);
    rho = r.robust ? huber_rho<R>(chi2, (R)r.delta) : chi2;
  }
  Acc<R> a;
  a.zero();
  a.add(rho);
  a = warp_sum_acc(a);
  const int lane = b.tid & 31, wid = b.tid >> 5, nw = b.nthr >> 5;
  if (lane == 0) sh[wid] = a.value();
  b.sync();
  if (wid == 0) {
    double t = (lane < nw) ? sh[lane] : 0.0;
    t = warp_sum(t);
    if (lane == 0) B.cost_part[b.id] = t;
  }
}



__device__ __forceinline__ void lm_begin_blk(const Bufs& B, const Blk& b, int ncost, double* sh) {
  double s = 0.0;
  for (int i = b.tid; i < ncost; i += b.nthr) s += B.cost_part[i];
  const double c = blk_sum(s, sh, b);
  if (b.tid == 0) {
    B.lm->current_chi = c;
    B.lm->initial_chi = c;
  }
}



// One LM trial's decision (optimization_algorithm_levenberg.cpp:113-141).
// The two partial sums run side by side (each in the order and tree of
// sum_partials), and thread 0 works on a register copy of the LM state,
// loaded before the sums and stored once at the end, so the decision is
// not a chain of dependent global loads.
// Returns, on the block's thread 0, whether another trial follows (0 or 1);
// -1 on every other thread.
__device__ __forceinline__ int lm_decide_blk(const Bufs& B, const Blk& b, int ncost, int nscale, double* sh) {
  LMState st;
  if (b.tid == 0) st = *B.lm;
  double c = 0.0, d = 0.0;
  for (int i = b.tid; i < ncost; i += b.nthr) c += B.cost_part[i];
  for (int i = b.tid; i < nscale; i += b.nthr) d += B.scale_part[i];
  const int lane = b.tid & 31, wid = b.tid >> 5, nw = b.nthr >> 5;
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    c += __shfl_xor_sync(0xffffffffu, c, o);
    d += __shfl_xor_sync(0xffffffffu, d, o);
  }
  if (lane == 0) {
    sh[wid] = c;
    sh[32 + wid] = d;
  }
  b.sync();
  if (wid != 0) return -1;
  c = (lane < nw) ? sh[lane] : 0.0;
  d = (lane < nw) ? sh[32 + lane] : 0.0;
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    c += __shfl_xor_sync(0xffffffffu, c, o);
    d += __shfl_xor_sync(0xffffffffu, d, o);
  }
  if (lane != 0) return -1;
  const double tempChi0 = c, scale0 = d;
  LMState* lm = &st;
  const double chi_before = lm->current_chi;
  double tempChi = tempChi0;
  if (!lm->solve_ok) tempChi = DBL_MAX;
  double rho = lm->current_chi - tempChi;
  double scale = scale0 + 1e-3;
  rho /= scale;
  const double lam_used = lm->lambda;
  const bool accepted = (rho > 0) && isfinite(tempChi);
  bool brk = false;
  if (accepted) {
    const double q = 2 * rho - 1;
    double alpha = 1. - q * q * q;
    alpha = fmin(alpha, 2. / 3.);
    const double sf = fmax(1. / 3., alpha);
    lm->lambda *= sf;
    lm->ni = 2;
    lm->current_chi = tempChi;
    lm->cur ^= 1;
  } else {
    lm->lambda *= lm->ni;
    lm->ni *= 2;
    if (!isfinite(lm->lambda)) brk = true;
  }
  if (lm->n_log < lm->max_log) {
    mcba_trial_log& L = B.log[lm->n_log];
    L.iteration = lm->iteration;
    L.trial = lm->trial;
    L.chi_before = chi_before;
    L.chi_after = tempChi;
    L.lambda = lam_used;
    L.scale = scale;
    L.rho = rho;
    L.accepted = accepted ? 1 : 0;
    L.solve_ok = lm->solve_ok;
  }
  lm->n_log++;
  lm->total_trials++;
  lm->temp_chi = tempChi;
  lm->rho = rho;
  lm->scale = scale;
  lm->last_accepted = accepted ? 1 : 0;
  if (!brk) lm->trial++;
  const bool more = !brk && rho < 0 && lm->trial < lm->max_trials &&
                    lm->total_trials < lm->max_iters * lm->max_trials;
  lm->trial_continue = more ? 1 : 0;
  if (!more) {
    if (lm->trial == lm->max_trials || rho == 0 || !isfinite(lm->lambda)) lm->terminate = 1;
    lm->iteration++;
  }
  // the next trial starts from a successful solve until the factorisation
  // says otherwise
  lm->solve_ok = 1;
  *B.lm = st;
  return more ? 1 : 0;
}

// activeRobustChi2 of the current (which = 0) or candidate (which = 1)
// state, one partial per CTA; the last CTA to finish then sums the partials
// (the fixed order and tree of a one-block launch) and takes the LM step:
// the initial cost (which = 0), or the trial's decision (which = 1), which
// in a graph also sets the trial loop's condition.
template <typename R>
__global__ void __launch_bounds__(256) k_cost_step(Bufs B, int E, int which, int nscale,
                                                   cudaGraphConditionalHandle h_trial, int in_graph) {
  __shared__ double sh[64];
  __shared__ int s_last;
  chain_wait();
  cost_blk<R>(B, grid_blk(), E, which, sh);
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(&B.done[0], 1) == (int)gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  if (threadIdx.x == 0) B.done[0] = 0;
  const Blk b{0, (int)threadIdx.x, (int)blockDim.x, 0};
  if (which == 0) {
    lm_begin_blk(B, b, (int)gridDim.x, sh);
  } else {
    const int more = lm_decide_blk(B, b, (int)gridDim.x, nscale, sh);
    if (more >= 0 && in_graph) cudaGraphSetConditional(h_trial, more ? 1u : 0u);
  }
}

// LM state at the start of a solve (OptimizationAlgorithmLevenberg members
// before iteration 0); in a graph it also arms the iteration loop.
__device__ __forceinline__ void lm_reset(LMState* lm, int max_trials, int max_log, int max_iters) {
  LMState z{};
  z.cur = 0;
  z.solve_ok = 1;
  z.max_trials = max_trials;
  z.max_log = max_log;
  z.max_iters = max_iters;
  z.lambda = -1;
  z.ni = 2;
  *lm = z;
}

__global__ void k_lm_reset(LMState* lm, int max_trials, int max_log, int max_iters,
                           cudaGraphConditionalHandle h_iter, int in_graph) {
  lm_reset(lm, max_trials, max_log, max_iters);
  if (in_graph) cudaGraphSetConditional(h_iter, max_iters > 0 ? 1u : 0u);
}

// End of one LM iteration (SparseOptimizer::optimize loop condition,
// sparse_optimizer.cpp:388): continue while not terminated and below the
// iteration count; the trial total is capped as a safety bound.
// The loop body has run outer_runs times; that count alone bounds the loop,
// whatever the trial loop did.
__device__ __forceinline__ bool iter_end(LMState* lm) {
  lm->outer_runs++;
  return !lm->terminate && lm->iteration < lm->max_iters && lm->outer_runs < lm->max_iters;
}

__global__ void k_iter_end(LMState* lm, cudaGraphConditionalHandle h_iter) {
  cudaGraphSetConditional(h_iter, iter_end(lm) ? 1u : 0u);
}

// Start of one LM iteration.  In the captured loop this also re-arms the
// trial loop: a conditional handle's default value is applied only when the
// whole graph is launched, so without this the inner WHILE would run zero
// times from the second iteration on.


// Zero the reduced camera matrix storage and put ones on the padding diagonal.
__device__ __forceinline__ void init_S_range(double* S, int ld, int n, size_t total, size_t i0, size_t step) {
  for (size_t i = i0; i < total; i += step) {
    const size_t r = i / ld, c = i % ld;
    S[i] = (r == c && (int)r >= n && (int)r < ld) ? 1.0 : 0.0;
  }
}

__global__ void k_init_S(double* S, int ld, int n, size_t total) {
  init_S_range(S, ld, n, total, blockIdx.x * (size_t)blockDim.x + threadIdx.x, (size_t)gridDim.x * blockDim.x);
}

__global__ void k_edge_chi2(const EdgeRec* recs, const float* obs, int E, StateView v, double* out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= E) return;
  const EdgeRec r = recs[j];
  const float o[3] = {obs[3 * (size_t)j], obs[3 * (size_t)j + 1], obs[3 * (size_t)j + 2]};
  double Pb[3], Pc[3], e[3], chi2;
  transform(r, v, Pb, Pc);
  edge_error<double>(r, o, v, Pc, e, chi2);
  out[j] = chi2;
}

// ------------------------------------------------ persistent window kernel --
// Many local-BA windows in one launch.  The grid is a set of thread-block
// clusters of C CTAs that stay resident; each cluster takes the next window
// from a device work queue (the host orders the windows by size, largest
// first) and runs its whole LM solve: the phases of a single solve's
// kernels, in the same order and over the same virtual blocks, with a
// cluster barrier between phases, and the reduced camera system factored by
// the cluster itself (the cluster LDL^T).  Sums therefore run in the same
// order as in a single solve, and the results are the single solve's.
//
// A CTA has the factorisation's 320 threads.  Phases written for 256-thread
// blocks run on warps 0-7 (named barrier 1); 128-thread blocks run two at a
// time on warps 0-3 and 4-7 (barriers 1 and 2); per-thread and per-warp
// work spreads over all ten warps of the cluster.
namespace cg = cooperative_groups;
constexpr int kWinThreads = chold::kThreads;

struct WinDesc {
  Bufs B;
  const double* qt0;  // initial state restored at the start of the solve
  const double* X0;
  int nchunk, Kf, Lf, E, n, npc, nblk, ld, ncost, nscale_pts, nscale_pose, K, NP, max_log;
  chold::Geo g;  // the factorisation's geometry for this launch's cluster size
};

struct WinArgs {
  const WinDesc* w;
  int nwin;
  int* queue;  // next window (reset to 0 before each launch)
  int iterations, max_trials;
  double tau;
};

template <typename R>
union WinShared {
  Acc<R> lin[kLinThreads / 32][32];
  Acc<R> se[6][kLinThreads / 32];
  Acc<R> asmb[kAsmGroups][36];
  double red[2][32];
  double dec[64];
};

__device__ __forceinline__ void cluster_barrier() { cg::this_cluster().sync(); }

// One window's LM solve by the calling cluster (the same control flow as
// the captured graph of add_lm_subgraph, with restore).
template <typename R>
__device__ void window_solve(const WinArgs& a, const WinDesc& d, int rank, int C, WinShared<R>& sh, double* dsm) {
  const Bufs& B = d.B;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int gt = rank * kWinThreads + tid, gn = C * kWinThreads;
  const int gw = rank * (kWinThreads / 32) + warp, gwn = C * (kWinThreads / 32);
  volatile LMState* vlm = B.lm;
  // blocks of 256 threads on warps 0-7; blocks of 128 threads two at a time
  auto run256 = [&](int nvb, auto&& body) {
    if (tid >= 256) return;
    for (int vb = rank; vb < nvb; vb += C) {
      const Blk b{vb, tid, 256, 1};
      body(b);
      b.sync();  // the block's shared memory is free for the next one
    }
  };
  auto run128 = [&](int nvb, auto&& body) {
    if (tid >= 256) return;
    const int half = tid >> 7;
    for (int base = 2 * rank; base < nvb; base += 2 * C) {
      const int vb = base + half;
      if (vb >= nvb) break;
      const Blk b{vb, tid & 127, 128, 1 + half};
      body(b, sh.red[half]);
      b.sync();
    }
  };

  // ---- prologue: restore the initial state (both halves), S padding, x = 0,
  //      LM state, initial cost
  for (int i = gt; i < d.K; i += gn) {
    double q[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) q[k] = d.qt0[8 * (size_t)i + k];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      B.pose_qt[0][8 * (size_t)i + k] = q[k];
      B.pose_qt[1][8 * (size_t)i + k] = q[k];
    }
    pose_lin_one(q, B.pd[0] + i, B.pf[0] + i);
    B.pd[1][i] = B.pd[0][i];
    B.pf[1][i] = B.pf[0][i];
  }
  for (int i = gt; i < d.NP; i += gn) {
    const double x0 = d.X0[3 * (size_t)i], x1 = d.X0[3 * (size_t)i + 1], x2 = d.X0[3 * (size_t)i + 2];
    for (int b = 0; b < 2; ++b) {
      B.Xd[b][3 * (size_t)i] = x0;
      B.Xd[b][3 * (size_t)i + 1] = x1;
      B.Xd[b][3 * (size_t)i + 2] = x2;
      B.Xf[b][i] = make_float4((float)x0, (float)x1, (float)x2, 0.f);
    }
  }
  init_S_range(B.S, d.ld, d.n, (size_t)(d.ld + kNB) * d.ld, gt, gn);
  for (int i = gt; i < d.n + 3 * d.Lf; i += gn) B.x[i] = 0.0;
  if (rank == 0 && tid == 0) lm_reset(B.lm, a.max_trials, d.max_log, a.iterations);
  cluster_barrier();
  run256(d.ncost, [&](const Blk& b) { cost_blk<R>(B, b, d.E, 0, sh.red[0]); });
  cluster_barrier();
  if (rank == 0 && tid < 256) lm_begin_blk(B, Blk{0, tid, 256, 1}, d.ncost, sh.red[0]);
  cluster_barrier();

  bool go = a.iterations > 0;
  for (int it = 0; go && it < a.iterations; ++it) {
    if (rank == 0 && tid == 0) iter_begin(B.lm);
    run256(d.nchunk, [&](const Blk& b) { linearize_blk<R>(B, b, sh.lin); });
    cluster_barrier();
    for (int i = gw; i < d.Kf; i += gwn) pose_reduce_warp<R>(B, d.Kf, i, lane);
    for (int l = gt; l < d.Lf; l += gn) point_reduce_thread<R>(B, d.Lf, l);
    cluster_barrier();
    if (vlm->iteration == 0) {
      const unsigned long long m = lambda_max_part<R>(B, d.Kf, d.Lf, gt, gn);
      if (lane == 0) atomicMax(&B.lm->lam_bits, m);
      cluster_barrier();
      if (rank == 0 && tid == 0) lambda_set(B.lm, a.tau);
    }
    cluster_barrier();
    for (int t = 0; t < a.max_trials; ++t) {
      if (d.Lf) {
        for (int l = gt; l < d.Lf; l += gn) point_dinv_one<R>(B, l);
        cluster_barrier();
      }
      if (d.Kf) {
        run256(d.nchunk, [&](const Blk& b) { schur_edge_blk<R>(B, b, sh.se); });
        cluster_barrier();
        for (int i = gw; i < d.npc; i += gwn) schur_pairs_warp<R>(B, i, lane);
        cluster_barrier();
        run256(d.nblk, [&](const Blk& b) { schur_assemble_blk<R>(B, b, d.ld, sh.asmb); });
        cluster_barrier();
        chold::ldlt_cluster_run(B.S, B.cws, B.x, &B.lm->solve_ok, d.g, dsm);
        chold::ldlt_cluster_retire(d.g, dsm, rank);
      }
      run128(d.nscale_pose + d.nscale_pts, [&](const Blk& b, double* shr) {
        update_blk<R>(B, b, d.Lf, d.n, d.Kf, d.nscale_pose, d.nscale_pts, shr);
      });
      cluster_barrier();
      run256(d.ncost, [&](const Blk& b) { cost_blk<R>(B, b, d.E, 1, sh.red[0]); });
      cluster_barrier();
      if (rank == 0 && tid < 256) lm_decide_blk(B, Blk{0, tid, 256, 1}, d.ncost, d.nscale_pts + d.nscale_pose, sh.dec);
      cluster_barrier();
      if (!vlm->trial_continue) break;
    }
    cluster_barrier();  // every thread has read trial_continue
    if (rank == 0 && tid == 0) iter_end(B.lm);
    cluster_barrier();
    go = !vlm->terminate && vlm->iteration < vlm->max_iters && vlm->outer_runs < vlm->max_iters;
  }
}

// kPerSM: CTAs per SM the launch is compiled for (1, or 2 with at most 96
// registers a thread and half the shared memory).
template <typename R, int kPerSM>
__global__ void __launch_bounds__(kWinThreads, kPerSM) k_windows(WinArgs a) {
  extern __shared__ __align__(16) double dsm[];
  __shared__ WinShared<R> sh;
  __shared__ int s_win;
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank(), C = (int)cl.num_blocks();
  for (int round = 0; round <= a.nwin; ++round) {
    if (rank == 0 && threadIdx.x == 0) s_win = atomicAdd(a.queue, 1);
    cl.sync();
    const int w = *cl.map_shared_rank(&s_win, 0);
    cl.sync();  // rank 0 overwrites s_win only after every CTA has read it
    if (w >= a.nwin) break;
    window_solve<R>(a, a.w[w], rank, C, sh, dsm);
  }
}

}  // namespace

// ----------------------------------------------------------- host side --
namespace {
struct Launch {
  int nchunk, Kf, Lf, Ec, E, n, npc, nblk, ld, nrows, ncost, nscale_pts, nscale_pose, tiles;
  int K, P, NP;
};
}  // namespace

class Solver {
 public:
  int device = 0;
  int precision = MCBA_PREC_FP64;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  // state
  DBuf<double> pose_qt[2], Xd[2], pose_qt0, Xd0;
  DBuf<PoseLinD> pd[2];
  DBuf<PoseLinF> pf[2];
  DBuf<float4> Xf[2];
  DBuf<CamD> cd;
  DBuf<CamF> cf;
  // structure
  DBuf<EdgeRec> recs, recs_all;
  DBuf<float> obs, obs_all;
  DBuf<int> chunk_begin, chunk_pose, pose_chunk_begin, pt_begin, canon_pose_h, canon_point_h, pchunk_begin,
      block_ab, block_chunk_begin, pose_canon_begin, pose_canon_list, free_pose_ids, free_point_ids;
  DBuf<int2> pairs;
  // numerics
  DBuf<char> rows, partials, Hll, bl, pdv, yq, ppart, qpart;
  DBuf<double> Hpp, bp, S, cws, dinv, x, cost_part, scale_part, chi2_out;
  DBuf<int> done;
  DBuf<LMState> lm;
  DBuf<mcba_trial_log> log;
  LMState* lm_host = nullptr;
  // pinned host buffers: the state upload and the read-backs after a solve
  // go through them as asynchronous copies, one synchronisation each
  struct Pinned {
    char* p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t n) {
      if (n <= cap && p) return cudaSuccess;
      if (p) cudaFreeHost(p);
      p = nullptr;
      cap = 0;
      const cudaError_t e = cudaMallocHost(&p, std::max<size_t>(n, 256));
      if (e == cudaSuccess) cap = std::max<size_t>(n, 256);
      return e;
    }
    void release() {
      if (p) cudaFreeHost(p);
      p = nullptr;
      cap = 0;
    }
  } h_up, h_rb;
  DeviceCompiler* compiler = nullptr;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  std::vector<cudaEvent_t> evpool;
  size_t evnext = 0;
  Launch L{};
  CholPlan chol;
  TiledChol tchol;  // side stream and events of the tiled solve (systems beyond the cluster solve)
  int chol_ld = -1, chol_n = -1;
  bool uploaded = false;
  int64_t launches = 0;
  int generation = 0;
  long long uid = 0;  // process-unique id (keys of cached batch graphs)
  // captured LM loop
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  int g_gen = -1, g_iters = -1, g_trials = -1, g_restore = -1;
  double g_tau = 0.0;
  // what a captured graph bakes in: launch sizes, buffer addresses, solve plan
  std::vector<char> g_sig;
  int64_t g_prologue = 0, g_per_iter = 0, g_per_trial = 0;

  void graph_release() {
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    gexec = nullptr;
    graph = nullptr;
    g_gen = -1;
  }

  cudaEvent_t next_event() {
    if (evnext == evpool.size()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      evpool.push_back(e);
    }
    return evpool[evnext++];
  }

  ~Solver() {
    cudaSetDevice(device);
    if (stream) cudaStreamSynchronize(stream);
    graph_release();
    chol_tiled_release(&tchol);
    DBuf<double>* ds[] = {&pose_qt[0], &pose_qt[1], &Xd[0], &Xd[1], &pose_qt0, &Xd0,
                          &Hpp, &bp, &S, &cws, &dinv, &x, &cost_part, &scale_part, &chi2_out};
    for (auto* d : ds) d->release();
    pd[0].release();
    pd[1].release();
    pf[0].release();
    pf[1].release();
    Xf[0].release();
    Xf[1].release();
    cd.release();
    cf.release();
    recs.release();
    recs_all.release();
    obs.release();
    obs_all.release();
    DBuf<int>* is[] = {&chunk_begin, &chunk_pose, &pose_chunk_begin, &pt_begin, &canon_pose_h, &canon_point_h,
                       &pchunk_begin, &block_ab, &block_chunk_begin, &pose_canon_begin, &pose_canon_list,
                       &free_pose_ids, &free_point_ids, &done};
    for (auto* d : is) d->release();
    pairs.release();
    DBuf<char>* cs[] = {&rows, &partials, &Hll, &bl, &pdv, &yq, &ppart, &qpart};
    for (auto* d : cs) d->release();
    lm.release();
    log.release();
    if (lm_host) cudaFreeHost(lm_host);
    h_up.release();
    h_rb.release();
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
    for (auto& e : evpool) cudaEventDestroy(e);
    if (compiler) compiler_destroy(compiler);
    if (own_stream && stream) cudaStreamDestroy(stream);
  }
};

#define CK(call)                                                                   \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess) {                                                       \
      if (err) *err = std::string(#call) + ": " + cudaGetErrorString(e_);          \
      return MCBA_ERR_CUDA;                                                        \
    }                                                                              \
  } while (0)

namespace {
// Idle solvers (library-owned stream) kept for the next handle on the same
// device and precision: device buffers, pinned staging, events, the stream
// and the captured graph are reused instead of being allocated again.  Up to
// 64 per key, so a batch of windows created and destroyed on every call
// (config 4: 64 local-BA windows) finds its workspaces again;
// mcba_release_cached frees them.
std::mutex g_pool_mu;
std::vector<Solver*> g_pool;
constexpr int kPoolPerKey = 64;
}  // namespace

Solver* solver_create(int device, int precision, void* stream, std::string* err) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    if (err) *err = "no CUDA device";
    return nullptr;
  }
  if (device < 0 || device >= n) {
    if (err) *err = "no CUDA device with that ordinal";
    return nullptr;
  }
  if (cudaSetDevice(device) != cudaSuccess) {
    if (err) *err = "cudaSetDevice failed";
    return nullptr;
  }
  if (!stream) {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    for (size_t i = 0; i < g_pool.size(); ++i)
      if (g_pool[i]->device == device && g_pool[i]->precision == precision) {
        Solver* s = g_pool[i];
        g_pool.erase(g_pool.begin() + (long)i);
        return s;
      }
  }
  Solver* s = new Solver();
  static std::atomic<long long> next_uid{1};
  s->uid = next_uid++;
  s->device = device;
  s->precision = precision;
  if (stream) {
    s->stream = (cudaStream_t)stream;
  } else {
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete s;
      if (err) *err = "cudaStreamCreate failed";
      return nullptr;
    }
    s->own_stream = true;
  }
  if (cudaMallocHost(&s->lm_host, sizeof(LMState)) != cudaSuccess) {
    delete s;
    if (err) *err = "cudaMallocHost failed";
    return nullptr;
  }
  for (auto& e : s->ev) cudaEventCreate(&e);
  return s;
}

void solver_destroy(Solver* s) {
  if (!s) return;
  if (s->own_stream) {
    cudaSetDevice(s->device);
    if (cudaStreamSynchronize(s->stream) == cudaSuccess) {
      s->uploaded = false;
      std::lock_guard<std::mutex> lk(g_pool_mu);
      int same = 0;
      for (Solver* q : g_pool) same += (q->device == s->device && q->precision == s->precision);
      if (same < kPoolPerKey) {
        g_pool.push_back(s);
        return;
      }
    }
  }
  delete s;
}

int solver_release_cached(int device) {
  std::vector<Solver*> drop;
  {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    for (size_t i = 0; i < g_pool.size();) {
      if (device < 0 || g_pool[i]->device == device) {
        drop.push_back(g_pool[i]);
        g_pool.erase(g_pool.begin() + (long)i);
      } else {
        ++i;
      }
    }
  }
  for (Solver* s : drop) delete s;
  return (int)drop.size();
}

bool solver_has_upload(const Solver* s) { return s && s->uploaded; }

namespace {

template <typename T>
cudaError_t up(DBuf<T>& d, const std::vector<T>& h, cudaStream_t st, int64_t& bytes) {
  cudaError_t e = d.ensure(h.size());
  if (e != cudaSuccess || h.empty()) return e;
  bytes += (int64_t)(h.size() * sizeof(T));
  return cudaMemcpyAsync(d.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, st);
}

void cam_to_dev(const HostCamera& c, CamD& d, CamF& f) {
  const double* q = c.T_cb.q;
  const double x = q[0], y = q[1], z = q[2], w = q[3];
  const double tx = 2 * x, ty = 2 * y, tz = 2 * z;
  const double Rm[9] = {1 - (ty * y + tz * z), ty * x - tz * w, tz * x + ty * w,
                        ty * x + tz * w,       1 - (tx * x + tz * z), tz * y - tx * w,
                        tz * x - ty * w,       tz * y + tx * w,       1 - (tx * x + ty * y)};
  for (int k = 0; k < 4; ++k) {
    d.K[k] = c.K[k];
    f.K[k] = c.K[k];
  }
  d.bf = c.bf;
  f.bf = c.bf;
  for (int k = 0; k < 9; ++k) {
    d.R[k] = Rm[k];
    f.R[k] = (float)Rm[k];
  }
  for (int k = 0; k < 3; ++k) {
    d.t[k] = c.T_cb.t[k];
    f.t[k] = (float)c.T_cb.t[k];
  }
}

// Both halves of the double-buffered state from the buffer-0 copy (or from
// the saved initial state), with the derived rotation matrices / float copies.
// Both halves of the state from the saved initial state (from_initial) or
// from half 0 just uploaded, which is then also saved as the initial state.
int spread_state(Solver* s, bool from_initial, std::string* err) {
  const Launch& L = s->L;
  if (L.K + L.NP == 0) return MCBA_OK;
  SpreadArgs a{};
  a.src_q = from_initial ? s->pose_qt0.p : s->pose_qt[0].p;
  a.src_x = from_initial ? s->Xd0.p : s->Xd[0].p;
  a.K = L.K;
  a.NP = L.NP;
  for (int b = 0; b < 2; ++b) {
    a.q[b] = s->pose_qt[b].p;
    a.x[b] = s->Xd[b].p;
    a.pd[b] = s->pd[b].p;
    a.pf[b] = s->pf[b].p;
    a.xf[b] = s->Xf[b].p;
  }
  a.keep_q = from_initial ? nullptr : s->pose_qt0.p;
  a.keep_x = from_initial ? nullptr : s->Xd0.p;
  const int n = L.K + L.NP;
  k_spread<<<std::min((n + 255) / 256, 1216), 256, 0, s->stream>>>(a);
  s->launches++;
  CK(cudaGetLastError());
  return MCBA_OK;
}

int upload_state(Solver* s, const HostProblem& hp, int U, int64_t& bytes, std::string* err) {
  const int K = (int)hp.poses.size();
  const int P = (int)hp.point_fixed.size();
  const int C = (int)hp.cams.size();
  // one pinned block: poses (8 per pose), points (3 per point, unary
  // constant points after them), cameras in both precisions
  const size_t nq = 8 * (size_t)std::max(K, 1), nx = 3 * (size_t)(P + U) + 3;
  const size_t oq = 0, ox = oq + nq * sizeof(double), ocd = ox + nx * sizeof(double);
  const size_t ocf = ocd + ((C * sizeof(CamD) + 15) & ~size_t(15)), total = ocf + C * sizeof(CamF);
  // the previous upload's copies may still read the block
  CK(cudaStreamSynchronize(s->stream));
  CK(s->h_up.ensure(total));
  double* q = reinterpret_cast<double*>(s->h_up.p + oq);
  double* X = reinterpret_cast<double*>(s->h_up.p + ox);
  CamD* cd = reinterpret_cast<CamD*>(s->h_up.p + ocd);
  CamF* cf = reinterpret_cast<CamF*>(s->h_up.p + ocf);
  std::fill(q, q + nq, 0.0);
  for (int k = 0; k < K; ++k) {
    for (int i = 0; i < 4; ++i) q[8 * k + i] = hp.poses[k].q[i];
    for (int i = 0; i < 3; ++i) q[8 * k + 4 + i] = hp.poses[k].t[i];
  }
  std::copy(hp.points.begin(), hp.points.end(), X);
  const size_t nu = std::min<size_t>(hp.u_Xw.size(), 3 * (size_t)U);
  std::copy(hp.u_Xw.begin(), hp.u_Xw.begin() + nu, X + 3 * (size_t)P);
  std::fill(X + 3 * (size_t)P + nu, X + nx, 0.0);
  for (int c = 0; c < C; ++c) cam_to_dev(hp.cams[c], cd[c], cf[c]);
  auto put = [&](void* dst, const void* src, size_t n) -> cudaError_t {
    bytes += (int64_t)n;
    return n ? cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, s->stream) : cudaSuccess;
  };
  CK(s->cd.ensure(std::max(C, 1)));
  CK(s->cf.ensure(std::max(C, 1)));
  CK(s->pose_qt[0].ensure(nq));
  CK(s->Xd[0].ensure(nx));
  CK(put(s->cd.p, cd, C * sizeof(CamD)));
  CK(put(s->cf.p, cf, C * sizeof(CamF)));
  CK(put(s->pose_qt[0].p, q, nq * sizeof(double)));
  CK(put(s->Xd[0].p, X, nx * sizeof(double)));
  const int NP = P + U;
  CK(s->pose_qt[1].ensure(nq));
  CK(s->Xd[1].ensure(nx));
  CK(s->pose_qt0.ensure(nq));
  CK(s->Xd0.ensure(nx));
  for (int b = 0; b < 2; ++b) {
    CK(s->pd[b].ensure(std::max(K, 1)));
    CK(s->pf[b].ensure(std::max(K, 1)));
    CK(s->Xf[b].ensure(std::max(NP, 1)));
  }
  s->L.K = K;
  s->L.P = P;
  s->L.NP = NP;
  return spread_state(s, false, err);
}

Bufs make_bufs(Solver* s) {
  Bufs B;
  for (int i = 0; i < 2; ++i) {
    B.pose_qt[i] = s->pose_qt[i].p;
    B.pd[i] = s->pd[i].p;
    B.pf[i] = s->pf[i].p;
    B.Xd[i] = s->Xd[i].p;
    B.Xf[i] = s->Xf[i].p;
  }
  B.cd = s->cd.p;
  B.cf = s->cf.p;
  B.recs = s->recs.p;
  B.obs = s->obs.p;
  B.chunk_begin = s->chunk_begin.p;
  B.chunk_pose = s->chunk_pose.p;
  B.pose_chunk_begin = s->pose_chunk_begin.p;
  B.pt_begin = s->pt_begin.p;
  B.canon_pose_h = s->canon_pose_h.p;
  B.canon_point_h = s->canon_point_h.p;
  B.pairs = s->pairs.p;
  B.pchunk_begin = s->pchunk_begin.p;
  B.block_ab = s->block_ab.p;
  B.block_chunk_begin = s->block_chunk_begin.p;
  B.pose_canon_begin = s->pose_canon_begin.p;
  B.pose_canon_list = s->pose_canon_list.p;
  B.free_pose_ids = s->free_pose_ids.p;
  B.free_point_ids = s->free_point_ids.p;
  B.rows = s->rows.p;
  B.partials = s->partials.p;
  B.Hpp = s->Hpp.p;
  B.bp = s->bp.p;
  B.bl = s->bl.p;
  B.Hll = reinterpret_cast<double*>(s->Hll.p);
  B.pdv = s->pdv.p;
  B.yq = s->yq.p;
  B.ppart = s->ppart.p;
  B.qpart = s->qpart.p;
  B.S = s->S.p;
  B.cws = s->cws.p;
  B.dinv = s->dinv.p;
  B.x = s->x.p;
  B.cost_part = s->cost_part.p;
  B.scale_part = s->scale_part.p;
  B.done = s->done.p;
  B.lm = s->lm.p;
  B.log = s->log.p;
  return B;
}

// Per-phase CUDA-event timing (profile option).
struct PhaseClock {
  Solver* s;
  bool on;
  struct Rec {
    int phase;
    cudaEvent_t a, b;
  };
  std::vector<Rec> pending;
  template <typename F>
  void run(int phase, F&& fn) {
    if (!on) {
      fn();
      return;
    }
    Rec r{phase, s->next_event(), s->next_event()};
    cudaEventRecord(r.a, s->stream);
    fn();
    cudaEventRecord(r.b, s->stream);
    pending.push_back(r);
  }
  // after a stream synchronisation
  void collect(SolveResult& out) {
    for (auto& r : pending) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
        out.ms_phase[r.phase] += ms;
        out.n_phase[r.phase]++;
      }
    }
    pending.clear();
    s->evnext = 0;
  }
};

// A kernel of the LM chain, launched so that it may start while the kernel
// before it on the stream finishes (see chain_wait).
template <typename... KArgs, typename... Args>
void launch_chain(void (*k)(KArgs...), int grid, int block, cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid, 1, 1);
  cfg.blockDim = dim3((unsigned)block, 1, 1);
  cfg.stream = st;
  cudaLaunchAttribute at;
  at.id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at.val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = &at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k, static_cast<KArgs>(args)...);
}

template <typename R>
void launch_linearize(Solver* s, const Bufs& B, const Launch& L, double tau, PhaseClock& pc,
                      cudaGraphConditionalHandle h_trial, int in_graph) {
  cudaStream_t st = s->stream;
  pc.run(MCBA_PHASE_LINEARIZE, [&] {
    launch_chain(k_linearize<R>, L.nchunk, kLinThreads, st, B, h_trial, in_graph);
    s->launches++;
  });
  pc.run(MCBA_PHASE_REDUCE, [&] {
    if (L.Kf || L.Lf) {
      const int npb = (L.Kf + 3) / 4;
      launch_chain(k_reduce<R>, npb + (L.Lf + 127) / 128, 128, st, B, L.Kf, L.Lf, npb, tau);
      s->launches++;
    }
  });
}

template <typename R>
void launch_trial(Solver* s, const Bufs& B, const Launch& L, PhaseClock& pc, cudaGraphConditionalHandle h_trial,
                  int in_graph) {
  cudaStream_t st = s->stream;
  if (L.Lf) {
    pc.run(MCBA_PHASE_SCHUR_EDGE, [&] {
      launch_chain(k_point_dinv<R>, (L.Lf + 127) / 128, 128, st, B, L.Lf);
      s->launches++;
    });
  }
  if (L.Kf) {
    pc.run(MCBA_PHASE_SCHUR_EDGE, [&] {
      launch_chain(k_schur_edge<R>, L.nchunk, kLinThreads, st, B);
      s->launches++;
    });
    pc.run(MCBA_PHASE_SCHUR_PAIRS, [&] {
      if (L.npc) {
        launch_chain(k_schur_pairs<R>, (L.npc + 7) / 8, 256, st, B, L.npc);
        s->launches++;
      }
    });
    pc.run(MCBA_PHASE_SCHUR_ASSEMBLE, [&] {
      launch_chain(k_schur_assemble<R>, L.nblk, 64 * kAsmGroups, st, B, L.ld);
      s->launches++;
    });
    pc.run(MCBA_PHASE_CHOLESKY, [&] {
      if (s->chol.ok) {
        chol_cluster_launch(s->chol, B.S, B.cws, L.ld, L.n, B.x, &B.lm->solve_ok, st);
        s->launches++;
        return;
      }
      long long nl = 0;
      chol_tiled_launch(s->tchol, B.S, B.cws, L.ld, L.n, B.x, &B.lm->solve_ok, st, &nl);
      s->launches += nl;
      // the tiled factorisation works in place and fills absent blocks in;
      // the next trial's assembly writes only the present blocks, so S
      // returns to zeros (identity padding) here
      const size_t total = (size_t)(L.ld + kNB) * L.ld;
      k_init_S<<<(int)std::min<size_t>((total + 255) / 256, 4096), 256, 0, st>>>(B.S, L.ld, L.n, total);
      s->launches++;
    });
  }
  pc.run(MCBA_PHASE_UPDATE, [&] {
    launch_chain(k_update<R>, L.nscale_pose + L.nscale_pts, 128, st, B, L.Lf, L.n, L.Kf, L.nscale_pose, L.nscale_pts);
    s->launches += 1;
  });
  pc.run(MCBA_PHASE_COST, [&] {
    launch_chain(k_cost_step<R>, L.ncost, 256, st, B, L.E, 1, L.nscale_pts + L.nscale_pose, h_trial, in_graph);
    s->launches += 1;
  });
}

template <typename R>
int alloc_numerics(Solver* s, std::string* err) {
  const Launch& L = s->L;
  const size_t rb = sizeof(R);
  const int nx = L.n + 3 * L.Lf;
  CK(s->rows.ensure(std::max<size_t>(1, (size_t)L.Ec * row_stride<R>() * rb)));
  const size_t ab = sizeof(Acc<R>);
  CK(s->partials.ensure(std::max<size_t>(1, (size_t)L.nchunk * 32 * ab)));
  CK(s->Hpp.ensure(std::max<size_t>(1, (size_t)L.Kf * 36)));
  CK(s->bp.ensure(std::max<size_t>(1, (size_t)L.Kf * 6)));
  CK(s->Hll.ensure(std::max<size_t>(1, (size_t)L.Lf * 6 * sizeof(double))));
  CK(s->pdv.ensure(std::max<size_t>(1, (size_t)L.Lf * kPdv * rb)));
  CK(s->bl.ensure(std::max<size_t>(1, (size_t)L.Lf * 3 * rb)));
  CK(s->yq.ensure(std::max<size_t>(1, (size_t)L.Ec * kYQ * rb)));
  CK(s->ppart.ensure(std::max<size_t>(1, (size_t)L.npc * 36 * ab)));
  CK(s->qpart.ensure(std::max<size_t>(1, (size_t)L.nchunk * 6 * ab)));
  CK(s->S.ensure((size_t)(L.ld + kNB) * L.ld));
  CK(s->cws.ensure(std::max(chol_cluster_ws_doubles(L.ld, L.n), chol_tiled_ws_doubles(L.ld))));
  CK(s->dinv.ensure(L.ld));
  CK(s->x.ensure(std::max(nx, 1)));
  CK(s->cost_part.ensure(L.ncost));
  CK(s->scale_part.ensure(L.nscale_pts + L.nscale_pose));
  CK(s->done.ensure(2));
  CK(s->lm.ensure(1));
  return MCBA_OK;
}

// Start of a solve: optional restore of the initial estimates, S padding,
// x = 0, LM state reset, initial activeRobustChi2.
template <typename R>
int launch_prologue(Solver* s, const Bufs& B, const RunOptions& o, bool restore, cudaGraphConditionalHandle h_iter,
                    int in_graph, std::string* err) {
  const Launch& L = s->L;
  cudaStream_t st = s->stream;
  if (restore) {
    const int r = spread_state(s, true, err);
    if (r) return r;
  }
  const int nx = L.n + 3 * L.Lf;
  const int max_log = std::max(1, o.iterations * o.max_trials);
  const size_t total = (size_t)(L.ld + kNB) * L.ld;
  k_init_S<<<(int)std::min<size_t>((total + 255) / 256, 4096), 256, 0, st>>>(B.S, L.ld, L.n, total);
  CK(cudaMemsetAsync(B.x, 0, std::max(nx, 1) * sizeof(double), st));
  CK(cudaMemsetAsync(B.done, 0, 2 * sizeof(int), st));
  k_lm_reset<<<1, 1, 0, st>>>(B.lm, o.max_trials, max_log, o.iterations, h_iter, in_graph);
  k_cost_step<R><<<L.ncost, 256, 0, st>>>(B, L.E, 0, 0, 0, 0);
  s->launches += 3;
  CK(cudaGetLastError());
  return MCBA_OK;
}

int capture_leaves(cudaStream_t st, std::vector<cudaGraphNode_t>& leaves, std::string* err) {
  cudaStreamCaptureStatus cs;
  const cudaGraphNode_t* deps = nullptr;
  const cudaGraphEdgeData* ed = nullptr;
  size_t nd = 0;
  CK(cudaStreamGetCaptureInfo(st, &cs, nullptr, nullptr, &deps, &ed, &nd));
  leaves.assign(deps, deps + nd);
  return MCBA_OK;
}

// Adds solver s's whole LM solve to graph G as an independent branch: the
// prologue, then
//   while (iterate) { linearise; while (trial) { Schur, Cholesky, update,
//   cost and decide }; end-of-iteration test }
// with both loop conditions set on the device (k_linearize re-arms the
// trial loop, k_cost_step's last CTA sets it, k_iter_end the outer one).
template <typename R>
int add_lm_subgraph(Solver* s, cudaGraph_t G, const RunOptions& o, bool restore, std::string* err) {
  const Launch& L = s->L;
  const Bufs B = make_bufs(s);
  cudaStream_t st = s->stream;
  PhaseClock pc{s, false, {}};
  cudaGraphConditionalHandle h_iter, h_trial;
  CK(cudaGraphConditionalHandleCreate(&h_iter, G, 0, cudaGraphCondAssignDefault));
  std::vector<cudaGraphNode_t> leaves;
  cudaGraph_t tmp;
  const int64_t l0 = s->launches;
  CK(cudaStreamBeginCaptureToGraph(st, G, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  int r = launch_prologue<R>(s, B, o, restore, h_iter, 1, err);
  if (r) {
    cudaStreamEndCapture(st, &tmp);
    return r;
  }
  r = capture_leaves(st, leaves, err);
  CK(cudaStreamEndCapture(st, &tmp));
  if (r) return r;
  s->g_prologue = s->launches - l0;

  cudaGraphNodeParams cp{};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h_iter;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t w_iter;
  CK(cudaGraphAddNode(&w_iter, G, leaves.data(), nullptr, leaves.size(), &cp));
  cudaGraph_t body_it = cp.conditional.phGraph_out[0];
  CK(cudaGraphConditionalHandleCreate(&h_trial, body_it, 1, cudaGraphCondAssignDefault));

  const int64_t l1 = s->launches;
  CK(cudaStreamBeginCaptureToGraph(st, body_it, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  launch_linearize<R>(s, B, L, o.tau, pc, h_trial, 1);
  r = capture_leaves(st, leaves, err);
  CK(cudaStreamEndCapture(st, &tmp));
  if (r) return r;

  cudaGraphNodeParams cp2{};
  cp2.type = cudaGraphNodeTypeConditional;
  cp2.conditional.handle = h_trial;
  cp2.conditional.type = cudaGraphCondTypeWhile;
  cp2.conditional.size = 1;
  cudaGraphNode_t w_trial;
  CK(cudaGraphAddNode(&w_trial, body_it, leaves.data(), nullptr, leaves.size(), &cp2));
  cudaGraph_t body_tr = cp2.conditional.phGraph_out[0];

  const int64_t l2 = s->launches;
  CK(cudaStreamBeginCaptureToGraph(st, body_tr, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  launch_trial<R>(s, B, L, pc, h_trial, 1);
  CK(cudaGetLastError());
  CK(cudaStreamEndCapture(st, &tmp));
  s->g_per_trial = s->launches - l2;

  CK(cudaStreamBeginCaptureToGraph(st, body_it, &w_trial, nullptr, 1, cudaStreamCaptureModeRelaxed));
  k_iter_end<<<1, 1, 0, st>>>(B.lm, h_iter);
  s->launches++;
  CK(cudaGetLastError());
  CK(cudaStreamEndCapture(st, &tmp));
  s->g_per_iter = (s->launches - l1) - s->g_per_trial;
  s->launches = l0;
  return MCBA_OK;
}

template <typename R>
int build_graph(Solver* s, const RunOptions& o, bool restore, std::string* err) {
  s->graph_release();
  cudaGraph_t G;
  CK(cudaGraphCreate(&G, 0));
  s->graph = G;
  const int r = add_lm_subgraph<R>(s, G, o, restore, err);
  if (r) return r;
  CK(cudaGraphInstantiate(&s->gexec, G, 0));
  s->g_gen = s->generation;
  s->g_iters = o.iterations;
  s->g_trials = o.max_trials;
  s->g_restore = restore ? 1 : 0;
  s->g_tau = o.tau;
  return MCBA_OK;
}

template <typename R>
int finish_run(Solver* s, const RunOptions& o, SolveResult& out, std::string* err) {
  const Launch& L = s->L;
  const int max_log = std::max(1, o.iterations * o.max_trials);
  out.initial_chi2 = s->lm_host->initial_chi;
  out.final_chi2 = s->lm_host->current_chi;
  out.lambda = s->lm_host->lambda;
  out.trials = s->lm_host->total_trials;
  const int nl = std::min(s->lm_host->n_log, max_log);
  out.log.resize(nl);
  // the trial log and the Hpp of the last linearisation (DumpCalculationGraph)
  // through the pinned read-back buffer, one synchronisation
  const size_t nh = (L.Kf && out.iterations > 0) ? (size_t)L.Kf * 36 : 0;
  const size_t blog = nl * sizeof(mcba_trial_log), bh = nh * sizeof(double);
  out.hpp.resize(nh);
  if (blog + bh) {
    CK(s->h_rb.ensure(blog + bh));
    if (blog) CK(cudaMemcpyAsync(s->h_rb.p, s->log.p, blog, cudaMemcpyDeviceToHost, s->stream));
    if (bh) CK(cudaMemcpyAsync(s->h_rb.p + blog, s->Hpp.p, bh, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    if (blog) std::memcpy(out.log.data(), s->h_rb.p, blog);
    if (bh) std::memcpy(out.hpp.data(), s->h_rb.p + blog, bh);
    out.d2h += (int64_t)(blog + bh);
  }
  return MCBA_OK;
}

template <typename R>
int run_lm_graph(Solver* s, const RunOptions& o, bool restore, SolveResult& out, std::string* err) {
  cudaStream_t stm = s->stream;
  const int max_log = std::max(1, o.iterations * o.max_trials);
  CK(s->log.ensure(max_log));
  if (!s->gexec || s->g_gen != s->generation || s->g_iters != o.iterations || s->g_trials != o.max_trials ||
      s->g_restore != (restore ? 1 : 0) || s->g_tau != o.tau) {
    const int r = build_graph<R>(s, o, restore, err);
    if (r) {
      s->graph_release();
      return r;
    }
  }
  CK(cudaEventRecord(s->ev[0], stm));
  CK(cudaGraphLaunch(s->gexec, stm));
  CK(cudaEventRecord(s->ev[1], stm));
  CK(cudaMemcpyAsync(s->lm_host, s->lm.p, sizeof(LMState), cudaMemcpyDeviceToHost, stm));
  out.d2h += sizeof(LMState);
  CK(cudaStreamSynchronize(stm));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, s->ev[0], s->ev[1]);
  out.ms_total = ms;
  out.iterations = s->lm_host->iteration;
  const int64_t iters_run = s->lm_host->iteration;
  s->launches += s->g_prologue + s->g_per_iter * iters_run + s->g_per_trial * s->lm_host->total_trials;
  return finish_run<R>(s, o, out, err);
}

template <typename R>
int run_lm(Solver* s, const RunOptions& o, bool restore, SolveResult& out, std::string* err) {
  const Launch& L = s->L;
  cudaStream_t stm = s->stream;
  const int iterations = o.iterations, max_trials = o.max_trials;
  const int max_log = std::max(1, iterations * max_trials);
  CK(s->log.ensure(max_log));
  Bufs B = make_bufs(s);
  PhaseClock pc{s, o.profile, {}};

  float ms_lin = 0.f;
  CK(cudaEventRecord(s->ev[0], stm));
  int r = 0;
  pc.run(MCBA_PHASE_COST, [&] { r = launch_prologue<R>(s, B, o, restore, 0, 0, err); });
  if (r) return r;
  int it = 0;
  bool stop = false;
  for (it = 0; it < iterations && !stop; ++it) {
    CK(cudaEventRecord(s->ev[2], stm));
    launch_linearize<R>(s, B, L, o.tau, pc, 0, 0);
    CK(cudaEventRecord(s->ev[3], stm));
    for (int t = 0; t < max_trials; ++t) {
      launch_trial<R>(s, B, L, pc, 0, 0);
      CK(cudaGetLastError());
      CK(cudaMemcpyAsync(s->lm_host, s->lm.p, sizeof(LMState), cudaMemcpyDeviceToHost, stm));
      out.d2h += sizeof(LMState);
      CK(cudaStreamSynchronize(stm));
      pc.collect(out);
      if (t == 0) {
        float m = 0.f;
        cudaEventElapsedTime(&m, s->ev[2], s->ev[3]);
        ms_lin += m;
      }
      if (!s->lm_host->trial_continue) break;
    }
    if (s->lm_host->terminate) stop = true;
  }
  CK(cudaEventRecord(s->ev[1], stm));
  CK(cudaMemcpyAsync(s->lm_host, s->lm.p, sizeof(LMState), cudaMemcpyDeviceToHost, stm));
  out.d2h += sizeof(LMState);
  CK(cudaStreamSynchronize(stm));
  pc.collect(out);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, s->ev[0], s->ev[1]);
  out.ms_total = ms;
  out.ms_linearize = ms_lin;
  out.iterations = it;
  return finish_run<R>(s, o, out, err);
}

}  // namespace

int solver_upload(Solver* s, const HostProblem& hp, const Structure* hst, StructureSizes* sizes, SolveResult& out,
                  std::string* err) {
  CK(cudaSetDevice(s->device));
  s->uploaded = false;
  int64_t bytes = 0;
  cudaStream_t stm = s->stream;
  StructureSizes z{};
  int r;
  if (hst) {
    const Structure& st = *hst;
    z.K = st.K;
    z.P = st.P;
    z.U = st.U;
    z.Kf = st.Kf;
    z.Lf = st.Lf;
    z.E = st.E;
    z.Ec = st.Ec;
    z.nchunk = (int)st.chunk_pose.size();
    z.npairs = (int)(st.pair_ij.size() / 2);
    z.nblk = (int)(st.block_ab.size() / 2);
    z.npc = (int)st.pchunk_block.size();
    if (sizes) *sizes = z;
    r = upload_state(s, hp, st.U, bytes, err);
    if (r) return r;
    CK(up(s->recs, st.recs, stm, bytes));
    CK(up(s->obs, st.obs, stm, bytes));
    CK(up(s->chunk_begin, st.chunk_begin, stm, bytes));
    CK(up(s->chunk_pose, st.chunk_pose, stm, bytes));
    CK(up(s->pose_chunk_begin, st.pose_chunk_begin, stm, bytes));
    CK(up(s->pt_begin, st.pt_begin, stm, bytes));
    CK(up(s->canon_pose_h, st.canon_pose_h, stm, bytes));
    CK(up(s->canon_point_h, st.canon_point_h, stm, bytes));
    CK(s->pairs.ensure(std::max<size_t>(1, st.pair_ij.size() / 2)));
    if (!st.pair_ij.empty()) {
      CK(cudaMemcpyAsync(s->pairs.p, st.pair_ij.data(), st.pair_ij.size() * sizeof(int32_t), cudaMemcpyHostToDevice, stm));
      bytes += st.pair_ij.size() * sizeof(int32_t);
    }
    CK(up(s->pchunk_begin, st.pchunk_begin, stm, bytes));
    CK(up(s->block_ab, st.block_ab, stm, bytes));
    CK(up(s->block_chunk_begin, st.block_chunk_begin, stm, bytes));
    CK(up(s->pose_canon_begin, st.pose_canon_begin, stm, bytes));
    CK(up(s->pose_canon_list, st.pose_canon_list, stm, bytes));
    CK(up(s->free_pose_ids, st.free_pose_ids, stm, bytes));
    CK(up(s->free_point_ids, st.free_point_ids, stm, bytes));
  } else {
    if (!s->compiler) s->compiler = compiler_create();
    r = compiler_phase1(s->compiler, hp, stm, &z, &bytes, err);
    if (r) return r;
    if (sizes) *sizes = z;
    if (z.Kf + z.Lf == 0 || z.E == 0) return MCBA_ERR_EMPTY;
    r = upload_state(s, hp, z.U, bytes, err);
    if (r) return r;
    CK(s->recs.ensure(z.E));
    CK(s->obs.ensure(3 * (size_t)z.E));
    CK(s->chunk_begin.ensure(z.nchunk + 1));
    CK(s->chunk_pose.ensure(z.nchunk + 1));
    CK(s->pose_chunk_begin.ensure(z.Kf + 1));
    CK(s->pt_begin.ensure(z.Lf + 1));
    CK(s->canon_pose_h.ensure(z.Ec + 1));
    CK(s->canon_point_h.ensure(z.Ec + 1));
    CK(s->pairs.ensure(std::max(z.npairs, 1)));
    CK(s->pchunk_begin.ensure(z.npc + 1));
    CK(s->block_ab.ensure(2 * (size_t)z.nblk + 2));
    CK(s->block_chunk_begin.ensure(z.nblk + 1));
    CK(s->pose_canon_begin.ensure(z.Kf + 1));
    CK(s->pose_canon_list.ensure(z.Ec + 1));
    CK(s->free_pose_ids.ensure(z.Kf + 1));
    CK(s->free_point_ids.ensure(z.Lf + 1));
    DeviceStructureOut o;
    o.recs = s->recs.p;
    o.obs = s->obs.p;
    o.chunk_begin = s->chunk_begin.p;
    o.chunk_pose = s->chunk_pose.p;
    o.pose_chunk_begin = s->pose_chunk_begin.p;
    o.pt_begin = s->pt_begin.p;
    o.canon_pose_h = s->canon_pose_h.p;
    o.canon_point_h = s->canon_point_h.p;
    o.pairs = s->pairs.p;
    o.pchunk_begin = s->pchunk_begin.p;
    o.block_ab = s->block_ab.p;
    o.block_chunk_begin = s->block_chunk_begin.p;
    o.pose_canon_begin = s->pose_canon_begin.p;
    o.pose_canon_list = s->pose_canon_list.p;
    o.free_pose_ids = s->free_pose_ids.p;
    o.free_point_ids = s->free_point_ids.p;
    r = compiler_phase2(s->compiler, o, stm, err);
    if (r) return r;
  }
  Launch& L = s->L;
  const int Kf = z.Kf, Lf = z.Lf, n = 6 * Kf;
  L.nchunk = z.nchunk;
  L.Kf = Kf;
  L.Lf = Lf;
  L.Ec = z.Ec;
  L.E = z.E;
  L.n = n;
  L.npc = z.npc;
  L.nblk = z.nblk;
  // systems beyond the cluster solve (384 unknowns) take the tiled solve
  L.ld = n > 384 ? chol_tiled_stride(n) : std::max(kNB, ((n + kNB - 1) / kNB) * kNB);
  L.tiles = L.ld / kNB;
  L.nrows = L.ld + 1;  // the b_schur row
  L.ncost = (z.E + 255) / 256;
  L.nscale_pts = std::max(1, (Lf + kPtsPerBlock - 1) / kPtsPerBlock);
  L.nscale_pose = std::max(1, (Kf + 127) / 128);
  if (L.ld > 4096) {
    if (err) *err = "reduced camera system above 4096 (682 free keyframes)";
    return MCBA_ERR_TOO_LARGE;
  }
  r = (s->precision == MCBA_PREC_MIXED) ? alloc_numerics<float>(s, err) : alloc_numerics<double>(s, err);
  if (r) return r;
  if (L.ld != s->chol_ld || L.n != s->chol_n) {
    s->chol = CholPlan();
    if (L.ld <= kClusterCholMaxLd && L.n > 0) chol_cluster_plan(L.ld, L.n, &s->chol);
    s->chol_ld = L.ld;
    s->chol_n = L.n;
  }
  if (!s->chol.ok && L.n > 0) {
    if (chol_tiled_setup(&s->tchol) != cudaSuccess) {
      if (err) *err = "tiled Cholesky set-up failed";
      return MCBA_ERR_CUDA;
    }
  }
  out.h2d += bytes;
  s->uploaded = true;
  // a captured LM graph stays valid while the launch sizes, the buffer
  // addresses and the solve plan are unchanged (everything else is read from
  // device memory when it runs)
  {
    const Bufs B = make_bufs(s);
    std::vector<char> sig(sizeof(Launch) + sizeof(Bufs) + 3 * sizeof(size_t));
    std::memcpy(sig.data(), &L, sizeof(Launch));
    std::memcpy(sig.data() + sizeof(Launch), &B, sizeof(Bufs));
    const size_t plan[3] = {(size_t)s->chol.ok, (size_t)s->chol.cluster, s->chol.smem_bytes};
    std::memcpy(sig.data() + sizeof(Launch) + sizeof(Bufs), plan, sizeof(plan));
    if (sig != s->g_sig) {
      s->g_sig.swap(sig);
      s->generation++;
    }
  }
  return MCBA_OK;
}

namespace {
// The graph of the last batch solved (independent branches, one per solver),
// kept while the same workspaces, uploads and options come back.
struct BatchGraph {
  std::vector<long long> uids;
  std::vector<int> gens;
  std::vector<const void*> logs;
  int iters = -1, trials = -1, device = -1;
  double tau = 0.0;
  cudaGraph_t g = nullptr;
  cudaGraphExec_t ge = nullptr;
  int64_t launches_prologue = 0;
  void release() {
    if (ge) cudaGraphExecDestroy(ge);
    if (g) cudaGraphDestroy(g);
    ge = nullptr;
    g = nullptr;
    uids.clear();
  }
};
std::mutex g_batch_mu;
BatchGraph g_batch;
}  // namespace

int solver_run_batch(Solver* const* ss, int n, const RunOptions& o, SolveResult* outs, double* ms_device,
                     std::string* err) {
  if (n <= 0) return MCBA_OK;
  for (int i = 0; i < n; ++i) {
    if (!ss[i] || !ss[i]->uploaded) {
      if (err) *err = "every problem of the batch must be prepared";
      return MCBA_ERR_INVALID;
    }
    if (ss[i]->device != ss[0]->device) {
      if (err) *err = "the problems of one batch must be on one device";
      return MCBA_ERR_INVALID;
    }
  }
  CK(cudaSetDevice(ss[0]->device));
  const int max_log = std::max(1, o.iterations * o.max_trials);
  for (int i = 0; i < n; ++i) CK(ss[i]->log.ensure(max_log));
  std::lock_guard<std::mutex> lk(g_batch_mu);
  std::vector<long long> uids(n);
  std::vector<int> gens(n);
  std::vector<const void*> logs(n);
  for (int i = 0; i < n; ++i) {
    uids[i] = ss[i]->uid;
    gens[i] = ss[i]->generation;
    logs[i] = ss[i]->log.p;
  }
  BatchGraph& bg = g_batch;
  if (!bg.ge || bg.uids != uids || bg.gens != gens || bg.logs != logs || bg.iters != o.iterations ||
      bg.trials != o.max_trials || bg.tau != o.tau || bg.device != ss[0]->device) {
    bg.release();
    CK(cudaGraphCreate(&bg.g, 0));
    for (int i = 0; i < n; ++i) {
      const int r = (ss[i]->precision == MCBA_PREC_MIXED) ? add_lm_subgraph<float>(ss[i], bg.g, o, true, err)
                                                          : add_lm_subgraph<double>(ss[i], bg.g, o, true, err);
      if (r) {
        bg.release();
        return r;
      }
    }
    CK(cudaGraphInstantiate(&bg.ge, bg.g, 0));
    bg.uids = uids;
    bg.gens = gens;
    bg.logs = logs;
    bg.iters = o.iterations;
    bg.trials = o.max_trials;
    bg.tau = o.tau;
    bg.device = ss[0]->device;
  }
  Solver* s0 = ss[0];
  cudaStream_t stm = s0->stream;
  CK(cudaEventRecord(s0->ev[0], stm));
  CK(cudaGraphLaunch(bg.ge, stm));
  CK(cudaEventRecord(s0->ev[1], stm));
  for (int i = 0; i < n; ++i) {
    CK(cudaMemcpyAsync(ss[i]->lm_host, ss[i]->lm.p, sizeof(LMState), cudaMemcpyDeviceToHost, stm));
    outs[i].d2h += sizeof(LMState);
  }
  CK(cudaStreamSynchronize(stm));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, s0->ev[0], s0->ev[1]);
  if (ms_device) *ms_device = ms;
  for (int i = 0; i < n; ++i) {
    Solver* s = ss[i];
    SolveResult& out = outs[i];
    out.ms_total = ms;
    out.iterations = s->lm_host->iteration;
    out.launches += s->g_prologue + s->g_per_iter * (int64_t)s->lm_host->iteration +
                    s->g_per_trial * (int64_t)s->lm_host->total_trials;
    const int r = (s->precision == MCBA_PREC_MIXED) ? finish_run<float>(s, o, out, err)
                                                    : finish_run<double>(s, o, out, err);
    if (r) return r;
  }
  return MCBA_OK;
}

namespace {
// The persistent window launch: descriptors and work queue on the device,
// the cluster size the autotuner chose for the batch, and the captured
// graph (queue reset + kernel), kept while the same workspaces, uploads and
// options come back.
struct PersistentBatch {
  std::vector<long long> uids;
  std::vector<int> gens;
  std::vector<const void*> logs;
  int iters = -1, trials = -1, device = -1, precision = -1;
  double tau = 0.0;
  int C = 0, nclusters = 0;
  int requested = -1;  // 0: the autotuner chose C; 4, 8, 16: the caller did
  int per_sm = 1;      // CTAs per SM the chosen kernel was compiled for
  size_t smem = 0;
  std::vector<std::pair<int, float>> tried;  // (CTAs per window, ms) of the autotuner
  DBuf<WinDesc> desc;
  DBuf<int> queue;
  cudaGraph_t g = nullptr;
  cudaGraphExec_t ge = nullptr;
  void release_graph() {
    if (ge) cudaGraphExecDestroy(ge);
    if (g) cudaGraphDestroy(g);
    ge = nullptr;
    g = nullptr;
  }
};
std::mutex g_pbatch_mu;
PersistentBatch g_pbatch;

// Descriptors of the windows (in launch order) for clusters of C CTAs, and
// the dynamic shared memory the launch needs; false when a window's reduced
// system does not fit the cluster factorisation.
template <typename R, int P>
bool window_descs(Solver* const* ss, const std::vector<int>& order, const RunOptions& o, int C,
                  std::vector<WinDesc>& out, size_t& smem, std::string* err) {
  int dev = 0, max_smem = 0, sm_smem = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaDeviceGetAttribute(&sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  if (P > 1) max_smem = std::min(max_smem, sm_smem / P - 1024);
  cudaFuncAttributes fa{};
  if (cudaFuncGetAttributes(&fa, k_windows<R, P>) != cudaSuccess) {
    cudaGetLastError();
    if (err) *err = "k_windows attributes";
    return false;
  }
  const size_t reserve = fa.sharedSizeBytes + 1024;
  out.clear();
  smem = 0;
  for (int i : order) {
    Solver* s = ss[i];
    const Launch& L = s->L;
    WinDesc d{};
    d.B = make_bufs(s);
    d.qt0 = s->pose_qt0.p;
    d.X0 = s->Xd0.p;
    d.nchunk = L.nchunk;
    d.Kf = L.Kf;
    d.Lf = L.Lf;
    d.E = L.E;
    d.n = L.n;
    d.npc = L.npc;
    d.nblk = L.nblk;
    d.ld = L.ld;
    d.ncost = L.ncost;
    d.nscale_pts = L.nscale_pts;
    d.nscale_pose = L.nscale_pose;
    d.K = L.K;
    d.NP = L.NP;
    d.max_log = std::max(1, o.iterations * o.max_trials);
    const int nb = (L.n + chold::kB - 1) / chold::kB;
    if (L.Kf && nb > chold::kMaxBlk) {
      if (err) *err = "a window's reduced camera system exceeds the persistent batch's limit (384 unknowns)";
      return false;
    }
    d.g = chold::make_geo(C, L.ld, L.n);
    const size_t bytes = L.Kf ? d.g.total() * sizeof(double) : 0;
    if (bytes + reserve > (size_t)max_smem) {
      if (err) *err = "a window's factorisation does not fit shared memory";
      return false;
    }
    smem = std::max(smem, bytes);
    out.push_back(d);
  }
  smem = std::max<size_t>(smem, 16);
  return true;
}

template <typename R, int P>
cudaError_t launch_windows(const PersistentBatch& pb, int nwin, const RunOptions& o, int C, int nclusters, size_t smem,
                           cudaStream_t st) {
  WinArgs a{pb.desc.p, nwin, pb.queue.p, o.iterations, o.max_trials, o.tau};
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(C * nclusters, 1, 1);
  cfg.blockDim = dim3(kWinThreads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr;
  attr.id = cudaLaunchAttributeClusterDimension;
  attr.val.clusterDim.x = C;
  attr.val.clusterDim.y = 1;
  attr.val.clusterDim.z = 1;
  cfg.attrs = &attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_windows<R, P>, a);
}

// Clusters of C CTAs that can be resident at once with `smem` bytes each
// (0 when the configuration cannot launch).
template <typename R, int P>
int window_clusters(int C, size_t smem) {
  int dev = 0, max_smem = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (cudaFuncSetAttribute(k_windows<R, P>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess ||
      cudaFuncSetAttribute(k_windows<R, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(C, 1, 1);
  cfg.blockDim = dim3(kWinThreads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute attr;
  attr.id = cudaLaunchAttributeClusterDimension;
  attr.val.clusterDim.x = C;
  attr.val.clusterDim.y = 1;
  attr.val.clusterDim.z = 1;
  cfg.attrs = &attr;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, k_windows<R, P>, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

template <typename R>
int run_windows(Solver* const* ss, int n, const RunOptions& o, SolveResult* outs, double* ms_device, int request,
                int* cluster_ctas, std::string* err) {
  Solver* s0 = ss[0];
  cudaStream_t stm = s0->stream;
  std::vector<long long> uids(n);
  std::vector<int> gens(n);
  std::vector<const void*> logs(n);
  for (int i = 0; i < n; ++i) {
    uids[i] = ss[i]->uid;
    gens[i] = ss[i]->generation;
    logs[i] = ss[i]->log.p;
  }
  PersistentBatch& pb = g_pbatch;
  const bool same = pb.ge && pb.uids == uids && pb.gens == gens && pb.logs == logs && pb.iters == o.iterations &&
                    pb.trials == o.max_trials && pb.tau == o.tau && pb.device == s0->device &&
                    pb.precision == s0->precision && pb.requested == request;
  if (!same) {
    pb.release_graph();
    // windows in descending size, so the largest start first
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
      const Launch &a = ss[x]->L, &b = ss[y]->L;
      return (long long)a.E + 4LL * a.npc * 32 > (long long)b.E + 4LL * b.npc * 32;
    });
    CK(pb.queue.ensure(1));
    CK(pb.desc.ensure(n));
    // autotuner: CTAs per window (cluster size) by timing the whole batch,
    // each candidate twice (the first run loads and warms up); a size the
    // caller asked for is the only candidate and is not timed
    pb.tried.clear();
    int bestC = 0, bestN = 0, bestP = 1;
    size_t bestSmem = 0;
    float best = 0.f;
    for (int P : {1, 2}) {
      if (request && P != 1) continue;
      for (int C : {4, 8, 16}) {
        if (request && C != request) continue;
        std::vector<WinDesc> d;
        size_t smem = 0;
        const bool ok = P == 1 ? window_descs<R, 1>(ss, order, o, C, d, smem, err)
                               : window_descs<R, 2>(ss, order, o, C, d, smem, err);
        if (!ok) {
          if (P == 1) return MCBA_ERR_INVALID;
          continue;  // the half-SM variant may not fit a large window's factorisation
        }
        const int ncl = P == 1 ? window_clusters<R, 1>(C, smem) : window_clusters<R, 2>(C, smem);
        if (ncl < 1) continue;
        const int nclusters = std::min(ncl, n);
        if (request) {
          bestC = C;
          bestN = nclusters;
          bestSmem = smem;
          break;
        }
        CK(cudaMemcpyAsync(pb.desc.p, d.data(), d.size() * sizeof(WinDesc), cudaMemcpyHostToDevice, stm));
        float ms = 0.f;
        for (int rep = 0; rep < 2; ++rep) {
          CK(cudaMemsetAsync(pb.queue.p, 0, sizeof(int), stm));
          CK(cudaEventRecord(s0->ev[0], stm));
          const cudaError_t le = P == 1 ? launch_windows<R, 1>(pb, n, o, C, nclusters, smem, stm)
                                        : launch_windows<R, 2>(pb, n, o, C, nclusters, smem, stm);
          CK(le);
          CK(cudaEventRecord(s0->ev[1], stm));
          CK(cudaStreamSynchronize(stm));
          CK(cudaEventElapsedTime(&ms, s0->ev[0], s0->ev[1]));
        }
        pb.tried.emplace_back(C * P, ms);
        if (!bestC || ms < best) {
          best = ms;
          bestC = C;
          bestN = nclusters;
          bestSmem = smem;
          bestP = P;
        }
      }
    }
    if (!bestC) {
      if (err) *err = "no cluster size can launch the persistent window kernel";
      return MCBA_ERR_CUDA;
    }
    std::vector<WinDesc> d;
    size_t smem = 0;
    if (!(bestP == 1 ? window_descs<R, 1>(ss, order, o, bestC, d, smem, err)
                     : window_descs<R, 2>(ss, order, o, bestC, d, smem, err)))
      return MCBA_ERR_INVALID;
    CK(cudaMemcpyAsync(pb.desc.p, d.data(), d.size() * sizeof(WinDesc), cudaMemcpyHostToDevice, stm));
    if (bestP == 1)
      window_clusters<R, 1>(bestC, smem);
    else
      window_clusters<R, 2>(bestC, smem);
    cudaGraph_t tmp;
    CK(cudaStreamBeginCapture(stm, cudaStreamCaptureModeRelaxed));
    cudaMemsetAsync(pb.queue.p, 0, sizeof(int), stm);
    if (bestP == 1)
      launch_windows<R, 1>(pb, n, o, bestC, bestN, bestSmem, stm);
    else
      launch_windows<R, 2>(pb, n, o, bestC, bestN, bestSmem, stm);
    CK(cudaStreamEndCapture(stm, &tmp));
    pb.g = tmp;
    CK(cudaGraphInstantiate(&pb.ge, pb.g, 0));
    pb.uids = uids;
    pb.gens = gens;
    pb.logs = logs;
    pb.iters = o.iterations;
    pb.trials = o.max_trials;
    pb.tau = o.tau;
    pb.device = s0->device;
    pb.precision = s0->precision;
    pb.C = bestC;
    pb.per_sm = bestP;
    pb.nclusters = bestN;
    pb.smem = bestSmem;
    pb.requested = request;
  }
  CK(cudaEventRecord(s0->ev[0], stm));
  CK(cudaGraphLaunch(pb.ge, stm));
  CK(cudaEventRecord(s0->ev[1], stm));
  for (int i = 0; i < n; ++i) {
    CK(cudaMemcpyAsync(ss[i]->lm_host, ss[i]->lm.p, sizeof(LMState), cudaMemcpyDeviceToHost, stm));
    outs[i].d2h += sizeof(LMState);
  }
  CK(cudaStreamSynchronize(stm));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, s0->ev[0], s0->ev[1]);
  if (ms_device) *ms_device = ms;
  if (cluster_ctas) *cluster_ctas = pb.C;
  for (int i = 0; i < n; ++i) {
    Solver* s = ss[i];
    SolveResult& out = outs[i];
    out.ms_total = ms;
    out.iterations = s->lm_host->iteration;
    out.launches += (i == 0) ? 1 : 0;  // one kernel for the whole batch
    const int r = finish_run<R>(s, o, out, err);
    if (r) return r;
  }
  return MCBA_OK;
}
}  // namespace

int solver_run_batch_persistent(Solver* const* ss, int n, const RunOptions& o, SolveResult* outs, double* ms_device,
                                int* cluster_ctas, std::string* err) {
  if (n <= 0) return MCBA_OK;
  const int request = cluster_ctas ? *cluster_ctas : 0;
  if (request != 0 && request != 4 && request != 8 && request != 16) {
    if (err) *err = "cluster_ctas must be 0 (autotune), 4, 8 or 16";
    return MCBA_ERR_INVALID;
  }
  for (int i = 0; i < n; ++i) {
    if (!ss[i] || !ss[i]->uploaded) {
      if (err) *err = "every problem of the batch must be prepared";
      return MCBA_ERR_INVALID;
    }
    if (ss[i]->device != ss[0]->device || ss[i]->precision != ss[0]->precision) {
      if (err) *err = "the problems of one persistent batch must share a device and a precision";
      return MCBA_ERR_INVALID;
    }
  }
  CK(cudaSetDevice(ss[0]->device));
  const int max_log = std::max(1, o.iterations * o.max_trials);
  for (int i = 0; i < n; ++i) CK(ss[i]->log.ensure(max_log));
  std::lock_guard<std::mutex> lk(g_pbatch_mu);
  return ss[0]->precision == MCBA_PREC_MIXED
             ? run_windows<float>(ss, n, o, outs, ms_device, request, cluster_ctas, err)
             : run_windows<double>(ss, n, o, outs, ms_device, request, cluster_ctas, err);
}

int solver_run(Solver* s, const RunOptions& o, bool restore, SolveResult& out, std::string* err) {
  if (!s->uploaded) {
    if (err) *err = "no problem uploaded";
    return MCBA_ERR_INVALID;
  }
  CK(cudaSetDevice(s->device));
  const int64_t l0 = s->launches;
  const bool graph = o.use_graph && !o.profile;
  int r;
  if (s->precision == MCBA_PREC_MIXED)
    r = graph ? run_lm_graph<float>(s, o, restore, out, err) : run_lm<float>(s, o, restore, out, err);
  else
    r = graph ? run_lm_graph<double>(s, o, restore, out, err) : run_lm<double>(s, o, restore, out, err);
  out.launches += s->launches - l0;
  return r;
}

int solver_download(Solver* s, HostProblem& hp, SolveResult& out, std::string* err) {
  CK(cudaSetDevice(s->device));
  const int K = (int)hp.poses.size(), P = (int)hp.point_fixed.size();
  const int cur = s->lm_host->cur;
  const size_t bq = 8 * (size_t)K * sizeof(double), bx = 3 * (size_t)P * sizeof(double);
  if (!(bq + bx)) return MCBA_OK;
  CK(s->h_rb.ensure(bq + bx));
  if (K) CK(cudaMemcpyAsync(s->h_rb.p, s->pose_qt[cur].p, bq, cudaMemcpyDeviceToHost, s->stream));
  if (P) CK(cudaMemcpyAsync(s->h_rb.p + bq, s->Xd[cur].p, bx, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  out.d2h += (int64_t)(bq + bx);
  if (P) std::memcpy(hp.points.data(), s->h_rb.p + bq, bx);
  const double* q = reinterpret_cast<const double*>(s->h_rb.p);
  for (int k = 0; k < K; ++k) {
    for (int i = 0; i < 4; ++i) hp.poses[k].q[i] = q[8 * k + i];
    for (int i = 0; i < 3; ++i) hp.poses[k].t[i] = q[8 * k + 4 + i];
  }
  return MCBA_OK;
}

int solver_edge_chi2(Solver* s, const HostProblem& hp, std::vector<double>& chi2, std::string* err) {
  CK(cudaSetDevice(s->device));
  int U = 0;
  for (size_t i = 0; i < hp.n_edges(); ++i)
    if (hp.e_type[i] == MCBA_EDGE_UNARY) ++U;
  int64_t bytes = 0;
  s->uploaded = false;  // the state buffers are reused below
  int r = upload_state(s, hp, U, bytes, err);
  if (r) return r;
  const int E = (int)hp.n_edges();
  const int P = (int)hp.point_fixed.size();
  std::vector<EdgeRec> recs(E);
  std::vector<float> obs(3 * (size_t)E);
  int u = 0;
  for (int i = 0; i < E; ++i) {
    EdgeRec& e = recs[i];
    e.pose = hp.e_pose[i];
    e.point = hp.e_type[i] == MCBA_EDGE_UNARY ? P + u++ : hp.e_point[i];
    e.pose_h = -1;
    e.point_h = -1;
    e.canon = -1;
    e.type = hp.e_type[i];
    e.cam = (uint8_t)hp.e_cam[i];
    e.robust = 0;
    e.dim = e.type == MCBA_EDGE_STEREO ? 3 : 2;
    e.info = hp.e_info[i];
    e.delta = hp.e_delta[i];
    for (int d = 0; d < 3; ++d) obs[3 * (size_t)i + d] = hp.e_obs[3 * (size_t)i + d];
  }
  cudaStream_t stm = s->stream;
  CK(up(s->recs_all, recs, stm, bytes));
  CK(up(s->obs_all, obs, stm, bytes));
  CK(s->chi2_out.ensure(std::max(E, 1)));
  StateView v;
  v.pd = s->pd[0].p;
  v.pf = s->pf[0].p;
  v.Xd = s->Xd[0].p;
  v.Xf = s->Xf[0].p;
  v.cd = s->cd.p;
  v.cf = s->cf.p;
  if (E) k_edge_chi2<<<(E + 255) / 256, 256, 0, stm>>>(s->recs_all.p, s->obs_all.p, E, v, s->chi2_out.p);
  CK(cudaGetLastError());
  chi2.resize(E);
  if (E) CK(cudaMemcpyAsync(chi2.data(), s->chi2_out.p, E * sizeof(double), cudaMemcpyDeviceToHost, stm));
  CK(cudaStreamSynchronize(stm));
  return MCBA_OK;
}

}  // namespace mcba

extern "C" int mcba_device_count(int* count) {
  if (!count) return MCBA_ERR_INVALID;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) n = 0;
  *count = n;
  return MCBA_OK;
}
