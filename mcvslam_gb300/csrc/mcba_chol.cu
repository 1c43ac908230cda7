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
// Cost model on GB300: an FP64 warp instruction occupies its SM
// sub-partition for ~64 cycles whatever the number of active lanes, an SM
// retires ~2 FP64 FMA per clock, and a distributed-shared-memory load waits
// ~2k cycles.  So the design (a) spreads the bulk FP64 work over the CTAs of
// one non-portable cluster (16), (b) keeps the pivot chain at five FP64
// instructions per pivot on four warps, one per sub-partition, (c) keeps
// the lanes of the bulk FP64 instructions busy and (d) pushes data to the
// CTAs that need it (remote stores, visible at the next cluster barrier)
// instead of pulling it:
//   * the lower triangle is cut into 16x16 tiles (tile t = i(i+1)/2 + j, the
//     right-hand side b is an extra block row); tile t lives in the shared
//     memory of CTA t mod C;
//   * step k: the owner of diagonal tile k has factored it and pushed it to
//     every CTA; the owners of the panel tiles (i,k) solve them against it,
//     one warp per two rows with shuffles, and push W = L D and L to the CTAs
//     whose share of the trailing update reads them; the trailing tiles are
//     dealt in contiguous ranges and updated in place at their owners;
//   * look-ahead: the owner of diagonal tile k+1 updates it first, factors it
//     and pushes it while the other CTAs finish the trailing update;
//   * the right-hand-side row leaves y = D^-1 L^-1 b; CTA 0 then solves
//     L^T x = y block row by block row, streaming row J-1 of L in while it
//     works on row J.

#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "mcba_chol.h"

namespace cg = cooperative_groups;

namespace mcba {
namespace {

constexpr int kB = 16;  // tile edge
constexpr int kThreads = 256;
constexpr int kTile = kB * kB;
constexpr int kPad = kB + 1;  // row stride of staged L tiles (conflict-free column reads)
constexpr int kPadTile = kB * kPad;

// Reciprocal of a pivot: rcp.approx.ftz.f64 (relative error ~1e-6), then one
// cubic Newton-Raphson step y (1 + e + e^2), e = 1 - d y, which leaves an
// error far below FP64 round-off.  Pivots whose reciprocal would leave the
// normal range take the IEEE division (integer test on the exponent field,
// so no FP64 comparison sits on the pivot chain).
__device__ __forceinline__ double recip_pivot(double d) {
  const unsigned ex = ((unsigned)(__double_as_longlong(d) >> 52)) & 0x7ffu;
  if (ex < 0x040u || ex > 0x7bfu) return 1.0 / d;
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(d));
  const double e = fma(-d, y, 1.0);
  const double p = fma(e, e, e);
  return fma(y, p, y);
}

__device__ __forceinline__ void bar_named(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

__host__ __device__ inline int tri_row(int t) {
  // largest a with a(a+1)/2 <= t
  int a = (int)((sqrtf(8.f * (float)t + 1.f) - 1.f) * 0.5f);
  while (a * (a + 1) / 2 > t) --a;
  while ((a + 1) * (a + 2) / 2 <= t) ++a;
  return a;
}

constexpr int kMaxBlk = 24;  // block rows handled by the cluster solve (n <= 384)

struct Geo {
  int C, nblk, ld, n, nslots;
  __host__ __device__ int nT0() const { return nblk * (nblk + 1) / 2; }
  __host__ __device__ int ntiles() const { return nT0() + nblk; }
  __host__ __device__ int tile(int i, int j) const { return i < nblk ? i * (i + 1) / 2 + j : nT0() + j; }
  __host__ __device__ int owner(int i, int j) const { return tile(i, j) % C; }
  __host__ __device__ int slot(int i, int j) const { return tile(i, j) / C; }
  // shared-memory layout (doubles), identical in every CTA
  __host__ __device__ size_t o_w() const { return (size_t)nslots * kTile; }          // W = L D of panel tiles
  __host__ __device__ size_t o_rd() const { return 2 * (size_t)nslots * kTile; }     // 1/d per diagonal slot
  __host__ __device__ size_t o_stw() const { return o_rd() + (size_t)nslots * kB; }  // pushed W tiles [nblk+1]
  __host__ __device__ size_t o_stl() const { return o_stw() + (size_t)(nblk + 1) * kTile; }  // pushed L [nblk]
  __host__ __device__ size_t o_lkk() const { return o_stl() + (size_t)nblk * kPadTile; }     // pushed L_kk, 1/d_k
  __host__ __device__ size_t o_t() const { return o_lkk() + kPadTile + kB; }          // backward-solve t [16 nblk]
  __host__ __device__ size_t o_flag() const { return o_t() + (size_t)kB * nblk; }
  __host__ __device__ size_t total() const { return o_flag() + 2; }
};

__device__ __forceinline__ void tile_ij(const Geo& g, int t, int& i, int& j) {
  const int nT0 = g.nT0();
  if (t >= nT0) {
    i = g.nblk;
    j = t - nT0;
    return;
  }
  i = tri_row(t);
  j = t - i * (i + 1) / 2;
}

// Trailing-update list of step k: tiles (i,j), k < j <= i < nblk, row by
// row, then the right-hand-side tiles (nblk, j), k < j < nblk.  Entry 0 is
// the next diagonal tile (k+1, k+1).
__device__ __forceinline__ void trail_ij(const Geo& g, int k, int L, int& i, int& j) {
  const int nrem = g.nblk - 1 - k;
  const int ntri = nrem * (nrem + 1) / 2;
  if (L >= ntri) {
    i = g.nblk;
    j = k + 1 + (L - ntri);
    return;
  }
  const int a = tri_row(L);
  i = k + 1 + a;
  j = k + 1 + (L - a * (a + 1) / 2);
}

// Entries [lo, hi) of the step-k list updated by CTA x, and the panel tiles
// it needs: W of block rows [rmin, rmax], L of block columns [cmin, cmax].
// The owner D of tile (k+1, k+1) takes entry 0 and factors that tile (about
// four tiles of work), then a reduced share; the other CTAs split the rest
// in contiguous ranges.
struct Need {
  int lo, hi, rmin, rmax, cmin, cmax;
};
__device__ __forceinline__ Need trail_need(const Geo& g, int k, int x) {
  const int C = g.C, nblk = g.nblk;
  const int nrem = nblk - 1 - k;
  const int m = nrem * (nrem + 1) / 2 + nrem;
  const int D = g.owner(k + 1, k + 1);
  const int q = (m + 4 + C - 1) / C;
  const int qD = min(max(0, q - 5), m - 1);
  const int rest = m - 1 - qD;
  const int per = (rest + C - 2) / (C - 1);
  const int idx = (x < D) ? x : x - 1;
  Need nd;
  nd.lo = (x == D) ? 1 : 1 + qD + min(rest, idx * per);
  nd.hi = (x == D) ? 1 + qD : 1 + qD + min(rest, (idx + 1) * per);
  nd.rmin = nblk + 1;
  nd.rmax = -1;
  nd.cmin = nblk;
  nd.cmax = -1;
  if (x == D) nd.rmin = nd.rmax = nd.cmin = nd.cmax = k + 1;
  if (nd.hi > nd.lo) {
    int i0, j0, i1, j1;
    trail_ij(g, k, nd.lo, i0, j0);
    trail_ij(g, k, nd.hi - 1, i1, j1);
    nd.rmin = min(nd.rmin, i0);
    nd.rmax = max(nd.rmax, i1);
    if (i0 == i1) {
      nd.cmin = min(nd.cmin, j0);
      nd.cmax = max(nd.cmax, j1);
    } else {
      nd.cmin = min(nd.cmin, k + 1);
      nd.cmax = max(nd.cmax, (i1 == nblk) ? nblk - 1 : i1);
    }
  }
  return nd;
}

// L D L^T of one 16x16 diagonal tile in place, by threads 0-127: strict
// lower part <- L, diagonal <- d, rd <- 1/d.  Entry (i, m), 1 <= m <= i,
// is updated by thread tid = i(i-1)/2 + m - 1 (120 threads, one FP64 FMA per
// pivot each); the pivot test runs once at the end on the diagonal.
__device__ void diag_ldlt(double* T, double* rd, int* fail) {
  const int tid = threadIdx.x;
  const bool has = tid < 120;
  const int a = tri_row(has ? tid : 0);
  const int ui = a + 1, um = (has ? tid : 0) - a * (a + 1) / 2 + 1;
  double* Tu = T + ui * kB + um;
  for (int j = 0; j < kB; ++j) {
    bar_named(1, 128);
    const double d = T[j * kB + j];
    const bool act = has && um > j;
    double prod = 0.0;
    if (act) prod = T[ui * kB + j] * T[um * kB + j];
    const double r = recip_pivot(d);
    if (tid == 0) rd[j] = r;
    if (act) *Tu = fma(-prod, r, *Tu);
  }
  bar_named(1, 128);
  if (tid < kB && !(T[tid * kB + tid] > 0.0)) *fail = 1;
  if (has) T[ui * kB + (um - 1)] *= rd[um - 1];
}

// D pushes the factorised diagonal tile (strict lower L) and 1/d into the
// staging area of every CTA of the cluster.
__device__ __forceinline__ void push_lkk(cg::cluster_group& cl, double* sm, const Geo& g, int k) {
  const int tid = threadIdx.x;
  const int s = g.slot(k, k);
  const double v = sm[(size_t)s * kTile + tid];
  const double rv = (tid < kB) ? sm[g.o_rd() + (size_t)s * kB + tid] : 0.0;
  for (int x = 0; x < g.C; ++x) {
    double* dst = cl.map_shared_rank(sm + g.o_lkk(), x);
    dst[(tid >> 4) * kPad + (tid & 15)] = v;
    if (tid < kB) dst[kPadTile + tid] = rv;
  }
}

__global__ void __launch_bounds__(kThreads) k_ldlt_cluster(const double* __restrict__ S, int ld, int n, double* x,
                                                           int* solve_ok, Geo g) {
  extern __shared__ double sm[];
  cg::cluster_group cl = cg::this_cluster();
  const int r = (int)cl.block_rank();
  const int C = g.C, nblk = g.nblk;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int* flag = reinterpret_cast<int*>(sm + g.o_flag());
  int* flag0 = cl.map_shared_rank(flag, 0);
  __shared__ Need s_need[16];
  __shared__ double s_x[kB];

  // owned tiles from the lower triangle of S (rows n..ld-1 of S are the
  // identity); right-hand-side tiles keep b in row 0
  for (int t = r; t < g.ntiles(); t += C) {
    int i, j;
    tile_ij(g, t, i, j);
    const int rr = tid >> 4, cc = tid & 15;
    double v;
    if (i < nblk)
      v = S[(size_t)(kB * i + rr) * ld + kB * j + cc];
    else
      v = (rr == 0) ? S[(size_t)ld * ld + kB * j + cc] : 0.0;
    sm[(size_t)(t / C) * kTile + tid] = v;
  }
  if (tid == 0) flag[0] = 0;
  cl.sync();
  if (g.owner(0, 0) == r) {
    if (tid < 128) diag_ldlt(sm + (size_t)g.slot(0, 0) * kTile, sm + g.o_rd() + (size_t)g.slot(0, 0) * kB, flag0);
    __syncthreads();
    push_lkk(cl, sm, g, 0);
  }
  cl.sync();

  double* stW = sm + g.o_stw();
  double* stL = sm + g.o_stl();
  for (int k = 0; k < nblk; ++k) {
    // ---- panel: tiles (i, k), k < i <= nblk, solved by their owners against
    //      the pushed diagonal block, then pushed to the CTAs of step k's
    //      trailing update that need them
    {
      int mine = 0;
      for (int i = k + 1; i <= nblk; ++i) mine += (g.owner(i, k) == r);
      if (mine) {
        if (k + 1 < nblk && tid < C) s_need[tid] = trail_need(g, k, tid);
        const double* Lkk = sm + g.o_lkk();
        // work items (panel tile, row pair); warp w takes items w, w + 8, ...
        int item = 0;
        for (int i = k + 1; i <= nblk; ++i) {
          if (g.owner(i, k) != r) continue;
          const int npair = (i < nblk) ? kB / 2 : 1;
          for (int p = 0; p < npair; ++p, ++item) {
            if ((item & 7) != warp) continue;
            const int s = g.slot(i, k);
            double* T = sm + (size_t)s * kTile;
            double* W = sm + g.o_w() + (size_t)s * kTile;
            const int row = 2 * p + (lane >> 4), c = lane & 15;
            double a = T[row * kB + c];
#pragma unroll
            for (int q = 0; q < kB - 1; ++q) {
              const double wq = __shfl_sync(0xffffffffu, a, (lane & 16) | q);
              if (c > q) a = fma(-wq, Lkk[c * kPad + q], a);
            }
            W[row * kB + c] = a;
            T[row * kB + c] = a * Lkk[kPadTile + c];
          }
        }
        __syncthreads();
        if (k + 1 < nblk) {
          const int rr = tid >> 4, cc = tid & 15;
          for (int i = k + 1; i <= nblk; ++i) {
            if (g.owner(i, k) != r) continue;
            const int s = g.slot(i, k);
            const double wv = sm[g.o_w() + (size_t)s * kTile + tid];
            const double lv = sm[(size_t)s * kTile + tid];
            for (int xx = 0; xx < C; ++xx) {
              const Need nd = s_need[xx];
              if (i >= nd.rmin && i <= nd.rmax)
                cl.map_shared_rank(stW, xx)[(size_t)i * kTile + tid] = wv;
              if (i < nblk && i >= nd.cmin && i <= nd.cmax)
                cl.map_shared_rank(stL, xx)[(size_t)i * kPadTile + rr * kPad + cc] = lv;
            }
          }
        }
      }
    }
    cl.sync();
    if (k == nblk - 1) break;

    // ---- trailing update of step k from the pushed panel tiles; the owner D
    //      of diagonal tile k+1 updates and factors it first (look-ahead)
    const Need nd = trail_need(g, k, r);
    const int D = g.owner(k + 1, k + 1);
    const int rr = tid >> 4, cc = tid & 15;
    if (r == D) {
      double* A = sm + (size_t)g.slot(k + 1, k + 1) * kTile;
      const double* wr = stW + (size_t)(k + 1) * kTile + rr * kB;
      const double* lc = stL + (size_t)(k + 1) * kPadTile + cc * kPad;
      double s0 = 0.0, s1 = 0.0;
#pragma unroll
      for (int q = 0; q < kB; q += 2) {
        s0 = fma(wr[q], lc[q], s0);
        s1 = fma(wr[q + 1], lc[q + 1], s1);
      }
      A[tid] -= s0 + s1;
      __syncthreads();
      const int s = g.slot(k + 1, k + 1);
      if (tid < 128) diag_ldlt(sm + (size_t)s * kTile, sm + g.o_rd() + (size_t)s * kB, flag0);
      __syncthreads();
      push_lkk(cl, sm, g, k + 1);
    }
    for (int L0 = nd.lo; L0 < nd.hi; L0 += 8) {
      double av[8];
      double* ap[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        ap[u] = nullptr;
        av[u] = 0.0;
        const int L = L0 + u;
        if (L < nd.hi) {
          int i, j;
          trail_ij(g, k, L, i, j);
          if (i < nblk || rr == 0) {
            ap[u] = cl.map_shared_rank(sm + (size_t)g.slot(i, j) * kTile, g.owner(i, j)) + tid;
            av[u] = *ap[u];
          }
        }
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int L = L0 + u;
        if (L >= nd.hi || !ap[u]) continue;
        int i, j;
        trail_ij(g, k, L, i, j);
        const double* wr = stW + (size_t)i * kTile + rr * kB;
        const double* lc = stL + (size_t)j * kPadTile + cc * kPad;
        double s0 = 0.0, s1 = 0.0;
#pragma unroll
        for (int q = 0; q < kB; q += 2) {
          s0 = fma(wr[q], lc[q], s0);
          s1 = fma(wr[q + 1], lc[q + 1], s1);
        }
        *ap[u] = av[u] - (s0 + s1);
      }
    }
    cl.sync();
  }

  // ---- backward solve L^T x = y (y: row 0 of the right-hand-side tiles) on
  //      CTA 0, which streams block row J-1 of L in while it works on row J
  // every CTA reads CTA 0's flag before any CTA may leave (a CTA's shared
  // memory must not be read remotely once it has exited)
  const int failed = *flag0;
  cl.sync();
  if (failed) {
    if (r == 0 && tid == 0) *solve_ok = 0;
    return;  // no CTA touches distributed shared memory after this point
  }
  if (r == 0) {
    double* t = sm + g.o_t();
    double* buf[2] = {stW, stL};  // row buffers (nblk tiles each)
    for (int e = tid; e < kB * nblk; e += kThreads) {
      const int I = e >> 4;
      t[e] = cl.map_shared_rank(sm + (size_t)g.slot(nblk, I) * kTile, g.owner(nblk, I))[e & 15];
    }
    for (int I = 0; I < nblk; ++I)  // row nblk-1
      buf[(nblk - 1) & 1][(size_t)I * kTile + tid] =
          cl.map_shared_rank(sm + (size_t)g.slot(nblk - 1, I) * kTile, g.owner(nblk - 1, I))[tid];
    __syncthreads();
    for (int J = nblk - 1; J >= 0; --J) {
      const double* Lr = buf[J & 1];
      // prefetch row J-1 into registers
      double pre[kMaxBlk];
#pragma unroll
      for (int I = 0; I < kMaxBlk; ++I)
        pre[I] = (J >= 1 && I <= J - 1)
                     ? cl.map_shared_rank(sm + (size_t)g.slot(J - 1, I) * kTile, g.owner(J - 1, I))[tid]
                     : 0.0;
      // x_J: unit upper solve L_JJ^T x_J = t_J, one warp
      if (warp == 0) {
        const int c = lane & 15;
        double tc = t[kB * J + c];
        const double* Ljj = Lr + (size_t)J * kTile;
#pragma unroll
        for (int q = kB - 1; q >= 0; --q) {
          const double xq = __shfl_sync(0xffffffffu, tc, q);
          if (c < q) tc = fma(-Ljj[q * kB + c], xq, tc);
        }
        if (lane < kB) {
          s_x[lane] = tc;
          if (kB * J + lane < n) x[kB * J + lane] = tc;
        }
      }
      __syncthreads();
      // t_I -= L_JI^T x_J, I < J
      for (int it = tid; it < kB * J; it += kThreads) {
        const int I = it >> 4, c = it & 15;
        const double* T = Lr + (size_t)I * kTile;
        double v0 = 0.0, v1 = 0.0;
#pragma unroll
        for (int q = 0; q < kB; q += 2) {
          v0 = fma(T[q * kB + c], s_x[q], v0);
          v1 = fma(T[(q + 1) * kB + c], s_x[q + 1], v1);
        }
        t[kB * I + c] -= v0 + v1;
      }
      if (J >= 1) {
        double* nb = buf[(J - 1) & 1];
#pragma unroll
        for (int I = 0; I < kMaxBlk; ++I)
          if (I <= J - 1) nb[(size_t)I * kTile + tid] = pre[I];
      }
      __syncthreads();
    }
  }
  cl.sync();  // every CTA keeps its shared memory until CTA 0 is done
}

Geo make_geo(int C, int ld, int n) {
  Geo g{};
  g.C = C;
  g.nblk = (n + kB - 1) / kB;
  g.ld = ld;
  g.n = n;
  g.nslots = (g.ntiles() + C - 1) / C;
  return g;
}

}  // namespace

int chol_cluster_plan(int ld, int n, CholPlan* plan) {
  plan->ok = false;
  if (n <= 0 || ld < kB * ((n + kB - 1) / kB) || (n + kB - 1) / kB > kMaxBlk) return 0;
  int dev = 0;
  cudaGetDevice(&dev);
  int max_smem = 0;
  cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const int reserve = 4096;  // static shared memory of the kernel
  if (cudaFuncSetAttribute(k_ldlt_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess ||
      cudaFuncSetAttribute(k_ldlt_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem - reserve) !=
          cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  for (int C : {16, 8}) {
    const Geo g = make_geo(C, ld, n);
    const size_t bytes = g.total() * sizeof(double);
    if (bytes + reserve > (size_t)max_smem) continue;
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
  const Geo g = make_geo(plan.cluster, ld, n);
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
  return cudaLaunchKernelEx(&cfg, k_ldlt_cluster, S, ld, n, x, solve_ok, g);
}

}  // namespace mcba
