// mcba_chol.cu -- FP64 solve of the reduced camera system on one
// thread-block cluster.
//
// LinearSolverEigen::solve (solvers/eigen/linear_solver_eigen.h:87-128)
// factors Hschur and solves for the pose update; a non-positive pivot makes
// the solve fail and leaves x untouched.  Here the factorisation is the
// square-root-free form S = L D L^T (unit lower L): the pivots d_j are the
// squares of the Cholesky diagonal, so "d_j <= 0" is the same failure test,
// and the solution is the same up to round-off.
//
// GB300 executes FP64 at ~1.6 FMA per clock per SM with ~64 cycles between
// dependent FP64 instructions, so the design keeps dependent FP64 chains
// short and spreads the bulk FP64 work over the CTAs of one cluster:
//   * 16-row block rows live in the shared memory of CTA (row block mod C);
//     other CTAs read and update them through distributed shared memory;
//   * per panel: the owner factors the 16x16 diagonal block (one pivot per
//     step, reciprocal by an FP32 estimate and one Newton-Raphson step
//     y <- y (2 - d y)), every CTA solves its own block rows against the
//     unit-lower diagonal block, then the trailing-update tiles are dealt
//     round-robin to all CTAs;
//   * the right-hand side rides along as an extra row, which leaves
//     y = D^-1 L^-1 b in it; the backward solve L^T x = y (unit diagonal, no
//     divisions) follows in the same kernel.

#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "mcba_chol.h"

namespace cg = cooperative_groups;

namespace mcba {
namespace {

constexpr int kB = 16;  // block size
constexpr int kThreads = 256;

// 1/d for d > 0: FP32 reciprocal, then one Newton-Raphson step in FP64
// (relative error ~ (2^-24)^2).
__device__ __forceinline__ double recip_newton(double d) {
  if (!(d > 1e-36 && d < 1e36)) return 1.0 / d;
  const double y = (double)__frcp_rn(__double2float_rn(d));
  const double e = fma(-d, y, 1.0);
  return fma(y, e, y);
}

struct Layout {
  int C, nblk, ld;  // ld: row stride of S; nblk block rows cover the n unknowns
  __host__ __device__ int owner(int j) const { return j % C; }
  __host__ __device__ int count(int o) const { return o < nblk ? (nblk - o + C - 1) / C : 0; }
  __host__ __device__ size_t block_off(int j) const {
    const int o = j % C, m = j / C;
    return (size_t)kB * kB * ((size_t)m * (o + 1) + (size_t)C * m * (m - 1) / 2);
  }
  __host__ __device__ size_t blocks_size(int o) const {
    const int m = count(o);
    return (size_t)kB * kB * ((size_t)m * (o + 1) + (size_t)C * m * (m - 1) / 2);
  }
  __host__ __device__ int w() const { return kB * nblk; }  // factorised width
  __host__ __device__ int b_owner() const { return nblk % C; }
  // CTA o: [block rows][b row (owner)][rdiag 16 per owned block][stage 2 x 256][t, x, flag (CTA 0)]
  __host__ __device__ size_t b_off(int o) const { return blocks_size(o); }
  __host__ __device__ size_t rdiag_off(int o) const { return b_off(o) + (o == b_owner() ? (size_t)w() : 0); }
  __host__ __device__ size_t stage_off(int o) const { return rdiag_off(o) + (size_t)kB * count(o); }
  __host__ __device__ size_t tx_off(int o) const { return stage_off(o) + 2 * kB * kB; }
  __host__ __device__ size_t total(int o) const { return tx_off(o) + (o == 0 ? 2 * (size_t)w() + 2 : 0); }
};

// First element of row `row` of block row `blk` in its owner's shared memory
// layout (blk == nblk: the b row).  The pointer is local; map it to the owner.
__device__ __forceinline__ double* row_ptr(double* sm, const Layout& Lo, int blk, int row) {
  if (blk == Lo.nblk) return sm + Lo.b_off(Lo.b_owner());
  return sm + Lo.block_off(blk) + (size_t)row * (kB * (blk + 1));
}

__global__ void __launch_bounds__(kThreads) k_ldlt_cluster(const double* __restrict__ S, int ld, int n, double* x,
                                                           int* solve_ok, Layout Lo) {
  extern __shared__ double sm[];
  cg::cluster_group cluster = cg::this_cluster();
  const int r = (int)cluster.block_rank();
  const int C = Lo.C, nblk = Lo.nblk, W = Lo.w();
  const int tid = threadIdx.x;
  double* rdiag = sm + Lo.rdiag_off(r);
  double* stage = sm + Lo.stage_off(r);
  double* t0 = cluster.map_shared_rank(sm + Lo.tx_off(0), 0);  // CTA 0: t[W], x[W], flag
  double* x0 = t0 + W;
  double* flag0 = x0 + W;

  // owned block rows and the b row, from the lower triangle of S (rows >= n
  // are the identity padding of S)
  for (int m = 0; m < Lo.count(r); ++m) {
    const int j = r + m * C;
    const int wj = kB * (j + 1);
    double* blk = sm + Lo.block_off(j);
    for (int idx = tid; idx < kB * wj; idx += kThreads) {
      const int rr = idx / wj, cc = idx % wj;
      blk[idx] = S[(size_t)(kB * j + rr) * ld + cc];
    }
  }
  if (r == Lo.b_owner())
    for (int c = tid; c < W; c += kThreads) sm[Lo.b_off(r) + c] = S[(size_t)ld * ld + c];
  if (r == 0 && tid == 0) *flag0 = 0.0;
  cluster.sync();

  for (int k = 0; k < nblk; ++k) {
    const int o = kB * k;
    // (1) L D L^T of the diagonal block by its owner: A[i][m] -= A[i][j] r_j A[m][j]
    if (Lo.owner(k) == r) {
      double* T = sm + Lo.block_off(k);
      const int wk = kB * (k + 1);
      double* rk = rdiag + (size_t)(k / C) * kB;
      __shared__ double rj;
      for (int j = 0; j < kB; ++j) {
        if (tid == 0) {
          const double d = T[j * wk + o + j];
          if (d <= 0.0) *flag0 = 1.0;
          const double y = recip_newton(d);
          rk[j] = y;
          rj = y;
        }
        __syncthreads();
        // pairs (i, m) with j < m <= i < 16: at most 120 updates
        if (tid < 120) {
          const int base = j + 1;
          int i = base, rem = tid;
          while (i < kB && rem >= i - base + 1) {
            rem -= i - base + 1;
            ++i;
          }
          if (i < kB) {
            const int m = base + rem;
            T[i * wk + o + m] -= (T[i * wk + o + j] * rj) * T[m * wk + o + j];
          }
        }
        __syncthreads();
      }
      // scale the strict lower part of the block to L: l_ij = a_ij r_j
      {
        const int i = tid / kB, j = tid % kB;
        if (i > j) T[i * wk + o + j] *= rk[j];
      }
      __syncthreads();
    }
    cluster.sync();
    // (2) every CTA: its block rows below the panel (and the b row) against
    //     the unit-lower diagonal block, then scaled by D^-1
    {
      const int ok = Lo.owner(k);
      const double* Tk = cluster.map_shared_rank(sm + Lo.block_off(k), ok);
      const double* rk = cluster.map_shared_rank(sm + Lo.rdiag_off(ok) + (size_t)(k / C) * kB, ok);
      __shared__ double Lkk[kB][kB + 1];
      __shared__ double rkk[kB];
      {
        const int i = tid / kB, j = tid % kB;
        Lkk[i][j] = Tk[i * (kB * (k + 1)) + o + j];
        if (tid < kB) rkk[tid] = rk[tid];
      }
      __syncthreads();
      const int first_m = (k >= r) ? (k - r) / C + 1 : 0;
      const int nb_own = max(0, Lo.count(r) - first_m);
      const int brow = (r == Lo.b_owner()) ? 1 : 0;
      const int nrows = kB * nb_own + brow;
      for (int c = 0; c < kB - 1; ++c) {
        for (int idx = tid; idx < nrows * kB; idx += kThreads) {
          const int row = idx / kB, cc = idx % kB;
          if (cc <= c) continue;
          double* p = (row < kB * nb_own) ? row_ptr(sm, Lo, r + (first_m + row / kB) * C, row % kB)
                                          : sm + Lo.b_off(r);
          p[o + cc] -= p[o + c] * Lkk[cc][c];
        }
        __syncthreads();
      }
      for (int idx = tid; idx < nrows * kB; idx += kThreads) {
        const int row = idx / kB, cc = idx % kB;
        double* p = (row < kB * nb_own) ? row_ptr(sm, Lo, r + (first_m + row / kB) * C, row % kB)
                                        : sm + Lo.b_off(r);
        p[o + cc] *= rkk[cc];
      }
      __syncthreads();
    }
    cluster.sync();
    // (3) trailing update A_ij -= L_ik D_k L_jk^T for k < j <= i (i == nblk: the
    //     b row), tiles dealt round-robin to the CTAs of the cluster
    {
      const int nrem = nblk - 1 - k;
      const int nlow = nrem * (nrem + 1) / 2;
      const int ntiles = nlow + nrem;
      const double* dk_src = cluster.map_shared_rank(sm + Lo.block_off(k), Lo.owner(k));
      __shared__ double dk[kB];
      if (tid < kB) dk[tid] = dk_src[tid * (kB * (k + 1)) + o + tid];
      __syncthreads();
      double* Li = stage;
      double* Lj = stage + kB * kB;
      for (int t = r; t < ntiles; t += C) {
        int bi, bj;
        if (t < nlow) {
          int a = 0, rem = t;
          while (rem >= a + 1) {
            rem -= a + 1;
            ++a;
          }
          bi = k + 1 + a;
          bj = k + 1 + rem;
        } else {
          bi = nblk;
          bj = k + 1 + (t - nlow);
        }
        const int rows_i = (bi == nblk) ? 1 : kB;
        const int oi = (bi == nblk) ? Lo.b_owner() : Lo.owner(bi);
        double* Ai = cluster.map_shared_rank(row_ptr(sm, Lo, bi, 0), oi);
        const int wi = (bi == nblk) ? W : kB * (bi + 1);
        const double* Aj = cluster.map_shared_rank(row_ptr(sm, Lo, bj, 0), Lo.owner(bj));
        const int wj = kB * (bj + 1);
        {
          const int rr = tid / kB, cc = tid % kB;
          Li[tid] = (rr < rows_i) ? Ai[(size_t)rr * wi + o + cc] * dk[cc] : 0.0;
          Lj[tid] = Aj[(size_t)rr * wj + o + cc];
        }
        __syncthreads();
        {
          const int rr = tid / kB, cc = tid % kB;
          if (rr < rows_i) {
            double s = 0.0;
#pragma unroll
            for (int q = 0; q < kB; ++q) s += Li[rr * kB + q] * Lj[cc * kB + q];
            Ai[(size_t)rr * wi + kB * bj + cc] -= s;
          }
        }
        __syncthreads();
      }
    }
    cluster.sync();
  }
  // y = D^-1 L^-1 b is the b row; backward solve L^T x = y one block row at a time
  if (r == Lo.b_owner())
    for (int c = tid; c < W; c += kThreads) t0[c] = sm[Lo.b_off(r) + c];
  cluster.sync();
  for (int I = nblk - 1; I >= 0; --I) {
    if (Lo.owner(I) == r) {
      const double* Ti = sm + Lo.block_off(I);
      const int wi = kB * (I + 1), o = kB * I;
      __shared__ double xi[kB];
      if (tid < 32) {
        const int lane = tid;
        double tc = (lane < kB) ? t0[o + lane] : 0.0;
        for (int c = kB - 1; c >= 0; --c) {
          const double xc = __shfl_sync(0xffffffffu, tc, c);
          if (lane < c) tc -= Ti[c * wi + o + lane] * xc;
          if (lane == c) {
            xi[c] = xc;
            x0[o + c] = xc;
          }
        }
      }
      __syncthreads();
      for (int col = tid; col < o; col += kThreads) {
        double s = 0.0;
#pragma unroll
        for (int rr = 0; rr < kB; ++rr) s += Ti[rr * wi + col] * xi[rr];
        t0[col] -= s;
      }
    }
    cluster.sync();
  }
  if (r == 0) {
    if (*flag0 != 0.0) {
      if (tid == 0) *solve_ok = 0;
    } else {
      for (int i = tid; i < n; i += kThreads) x[i] = x0[i];
    }
  }
}

Layout make_layout(int C, int ld, int n) { return Layout{C, (n + kB - 1) / kB, ld}; }

}  // namespace

int chol_cluster_plan(int ld, int n, CholPlan* plan) {
  plan->ok = false;
  if (n <= 0 || ld < n) return 0;
  int dev = 0;
  cudaGetDevice(&dev);
  int max_smem = 0;
  cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (cudaFuncSetAttribute(k_ldlt_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess ||
      cudaFuncSetAttribute(k_ldlt_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem - 8192) !=
          cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  for (int C : {16, 8}) {
    const Layout Lo = make_layout(C, ld, n);
    size_t need = 0;
    for (int o = 0; o < C; ++o) need = std::max(need, Lo.total(o));
    const size_t bytes = need * sizeof(double);
    if (bytes + 8192 > (size_t)max_smem) continue;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(C, 1, 1);
    cfg.blockDim = dim3(kThreads, 1, 1);
    cfg.dynamicSmemBytes = bytes;
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeClusterDimension;
    attr.val.clusterDim.x = C;
    attr.val.clusterDim.y = 1;
    attr.val.clusterDim.z = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, k_ldlt_cluster, &cfg) != cudaSuccess || nclusters < 1) {
      cudaGetLastError();
      continue;
    }
    plan->ok = true;
    plan->cluster = C;
    plan->smem_bytes = bytes;
    return 1;
  }
  return 0;
}

cudaError_t chol_cluster_launch(const CholPlan& plan, const double* S, int ld, int n, double* x, int* solve_ok,
                                cudaStream_t st) {
  const Layout Lo = make_layout(plan.cluster, ld, n);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(plan.cluster, 1, 1);
  cfg.blockDim = dim3(kThreads, 1, 1);
  cfg.dynamicSmemBytes = plan.smem_bytes;
  cfg.stream = st;
  cudaLaunchAttribute attr;
  attr.id = cudaLaunchAttributeClusterDimension;
  attr.val.clusterDim.x = plan.cluster;
  attr.val.clusterDim.y = 1;
  attr.val.clusterDim.z = 1;
  cfg.attrs = &attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_ldlt_cluster, S, ld, n, x, solve_ok, Lo);
}

}  // namespace mcba
