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
// Cost model on GB300 (measured): a dependent FP64 FMA takes 64 cycles and an
// SM retires ~1.6 FP64 FMA per clock; a cluster barrier costs ~400 cycles;
// distributed-shared-memory stores move only ~13 B per clock per SM, while
// the 129 MB L2 serves an SM several times faster.  So the bulk FP64 work is
// spread over the CTAs of one 16-CTA cluster, the barriers are the cluster's,
// and the tiles themselves live in an L2-resident workspace (same shape as
// S; S is only read), so any CTA can update any tile:
//   * the lower triangle is cut into 16x16 tiles, the right-hand side b is an
//     extra block row;
//   * step k, panel: the CTA D(k+1) chosen for diagonal tile (k+1, k+1)
//     solves panel tile (k+1, k) itself (keeping W and L of it in shared
//     memory) and prefetches tile (k+1, k+1); the other panel tiles (i, k),
//     k+1 < i <= nblk, are spread over the other CTAs.  Each is solved
//     against L_kk and 1/d_k, and W_ik = L_ik D_k is written over it (lower
//     tile (i, k)) and L_ik into the upper tile (k, i); the right-hand-side
//     tile leaves W in row ld and y_k = D^-1 L^-1 b in row ld + 2;
//   * step k, update: D(k+1) applies step k to its diagonal tile, factors it
//     (the pivot chain alone on one warp) and writes L, d and 1/d (row
//     ld + 1); the other trailing tiles are dealt in contiguous ranges, D
//     taking a reduced share after its factorisation.  Each CTA stages the
//     panel rows and columns its range needs in shared memory and keeps eight
//     tiles (and eight L2 loads per thread) in flight;
//   * CTA 0 then solves L^T x = y block row by block row, staging the next
//     block row while warp 0 works on the current one.
// Failure (a pivot <= 0) clears *solve_ok in global memory; CTA 0 reads it
// after the last barrier and then leaves x untouched.  No CTA reads another
// CTA's shared memory, so CTAs may leave as soon as they are done.

#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "mcba_chol.h"

namespace mcba {
namespace {

namespace cg = cooperative_groups;

constexpr int kB = 16;  // tile edge
constexpr int kThreads = 256;
constexpr int kTile = kB * kB;
constexpr int kPad = kB + 1;  // row stride of staged L tiles (conflict-free column reads)
constexpr int kPadTile = kB * kPad;
constexpr int kMaxBlk = 24;  // block rows handled by the cluster solve (n <= 384)

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

struct Geo {
  int C, nblk, ld, n;
  // shared-memory layout (doubles), identical in every CTA
  __host__ __device__ size_t o_stw() const { return 0; }                                      // W rows [nblk+1]
  __host__ __device__ size_t o_stl() const { return (size_t)(nblk + 1) * kTile; }             // L [nblk]
  __host__ __device__ size_t o_lkk() const { return o_stl() + (size_t)nblk * kPadTile; }     // L_kk, 1/d_k
  __host__ __device__ size_t o_diag() const { return o_lkk() + kPadTile + kB; }  // D's tile, 1/d, squares
  __host__ __device__ size_t o_t() const { return o_diag() + kTile + 2 * kB; }               // backward-solve t
  __host__ __device__ size_t total() const { return o_t() + (size_t)kB * nblk; }
  // backward solve: two block rows of L, over the (then idle) staging areas
  __host__ __device__ size_t o_buf() const { return o_stw(); }
  // the CTA that factors diagonal tile k
  __host__ __device__ int diag_cta(int k) const { return (k * 7 + 3) % C; }
};

// Workspace (row stride ld, ld + 32 rows): the lower triangle of S, updated in
// place; W_ik over the lower tile (i, k) once step k is done, L_ik in the
// upper tile (k, i) stored as its own 16x16 array, L_kk and d in the diagonal
// tile; right-hand side: b then W in row ld, 1/d in row ld + 1, y in row
// ld + 2.
__device__ __forceinline__ double* ws_lower(double* ws, int ld, int i, int k) {
  return ws + (size_t)(kB * i) * ld + kB * k;
}
__device__ __forceinline__ double* ws_upper(double* ws, int ld, int j, int k) {
  return ws + (size_t)(kB * k) * ld + kB * j;
}
// element (rr, cc) of tile (i, j) of the updated matrix; block row nblk is b
__device__ __forceinline__ double* ws_tile(double* ws, int ld, int nblk, int i, int j, int rr, int cc) {
  return (i < nblk) ? ws_lower(ws, ld, i, j) + (size_t)rr * ld + cc : ws + (size_t)ld * ld + kB * j + cc;
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
// D takes entry 0 (the next diagonal tile, which it then factors: about four
// tiles of work) and then a reduced share; the other CTAs split the rest in
// contiguous ranges.
struct Need {
  int lo, hi, rmin, rmax, cmin, cmax;
};
__device__ __forceinline__ Need trail_need(const Geo& g, int k, int x) {
  const int C = g.C, nblk = g.nblk;
  const int nrem = nblk - 1 - k;
  const int m = nrem * (nrem + 1) / 2 + nrem;
  const int D = g.diag_cta(k + 1);
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
  if (nd.hi > nd.lo) {
    int i0, j0, i1, j1;
    trail_ij(g, k, nd.lo, i0, j0);
    trail_ij(g, k, nd.hi - 1, i1, j1);
    nd.rmin = i0;
    nd.rmax = i1;
    if (i0 == i1) {
      nd.cmin = j0;
      nd.cmax = j1;
    } else {
      nd.cmin = k + 1;
      nd.cmax = (i1 == nblk) ? nblk - 1 : i1;
    }
  }
  return nd;
}

// Stage W_{i,k} for rows [r0, r1] and L_{j,k} for columns [c0, c1] from the
// workspace, eight tiles per round so that each thread has eight L2 loads in
// flight.
__device__ void stage_panel(const Geo& g, double* ws, int k, int r0, int r1, int c0, int c1, double* stW,
                            double* stL) {
  const int tid = threadIdx.x, rr = tid >> 4, cc = tid & 15;
  const int nblk = g.nblk, ld = g.ld;
  const int nr = max(0, r1 - r0 + 1), nc = max(0, c1 - c0 + 1), nt = nr + nc;
  for (int base = 0; base < nt; base += 8) {
    double v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      v[u] = 0.0;
      const int e = base + u;
      if (e < nr) {
        const int i = r0 + e;
        if (i < nblk || rr == 0) v[u] = __ldcg(ws_tile(ws, ld, nblk, i, k, rr, cc));
      } else if (e < nt) {
        v[u] = __ldcg(ws_upper(ws, ld, c0 + e - nr, k) + (size_t)rr * ld + cc);
      }
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int e = base + u;
      if (e < nr)
        stW[(size_t)(r0 + e) * kTile + tid] = v[u];
      else if (e < nt)
        stL[(size_t)(c0 + e - nr) * kPadTile + rr * kPad + cc] = v[u];
    }
  }
}

// L D L^T of one 16x16 diagonal tile in place: strict lower part <- L,
// diagonal <- d, rd <- 1/d.  The pivot chain runs alone on warp 0 (its own
// sub-partition, so no other FP64 work queues in front of it): from r_j it
// forms d_{j+1} = a_{j+1,j+1} - a_{j+1,j}^2 r_j itself and takes its
// reciprocal, while warps 1-3 and 5-7 apply pivot j to the other entries
// (entry (i, m), 1 <= m <= i, on update thread u = i(i-1)/2 + m - 1; the
// diagonal entry skips the pivot that warp 0 applies, and entry (i, i-1)
// leaves its square in sq[i] once final).  One named barrier per pivot;
// warp 4 takes no part.  The arithmetic is the plain right-looking LDL^T.
__device__ void diag_ldlt(double* T, double* rd, double* sq, int* solve_ok) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  constexpr int kPart = 224;  // warps 0-3 and 5-7
  if (warp == 0) {
    double r = recip_pivot(T[0]);
    if (lane == 0) rd[0] = r;
    for (int j = 0; j < kB; ++j) {
      bar_named(1, kPart);  // pivot j-1 applied everywhere, r_j published
      if (j + 1 < kB) {
        const double s = (j == 0) ? T[kB] * T[kB] : sq[j + 1];
        const double d = fma(-s, r, T[(j + 1) * kB + j + 1]);
        if (lane == 0) T[(j + 1) * kB + j + 1] = d;
        r = recip_pivot(d);
        if (lane == 0) rd[j + 1] = r;
      }
    }
    bar_named(1, kPart);
  } else {
    const int u = (warp < 4) ? (warp - 1) * 32 + lane : (warp - 2) * 32 + lane;
    const bool has = u < 120;
    const int a = tri_row(has ? u : 0);
    const int ui = a + 1, um = (has ? u : 0) - a * (a + 1) / 2 + 1;
    double* Tu = T + ui * kB + um;
    for (int j = 0; j < kB; ++j) {
      bar_named(1, kPart);
      if (has && um > j && !(ui == um && um == j + 1)) {
        const double prod = T[ui * kB + j] * T[um * kB + j];
        const double v = fma(-prod, rd[j], *Tu);
        *Tu = v;
        if (um == ui - 1 && j == um - 1) sq[ui] = v * v;
      }
    }
    bar_named(1, kPart);
    if (has) T[ui * kB + (um - 1)] *= rd[um - 1];
  }
  if (tid < kB && !(T[tid * kB + tid] > 0.0)) *solve_ok = 0;
}

// Factor the diagonal tile held in shared memory T and publish L, d, 1/d.
__device__ void factor_publish(const Geo& g, double* ws, double* T, int k, int* solve_ok) {
  const int tid = threadIdx.x, rr = tid >> 4, cc = tid & 15;
  double* rd = T + kTile;
  double* sq = rd + kB;
  if ((tid >> 5) != 4) diag_ldlt(T, rd, sq, solve_ok);
  __syncthreads();
  ws_lower(ws, g.ld, k, k)[(size_t)rr * g.ld + cc] = T[tid];
  if (tid < kB) ws[(size_t)(g.ld + 1) * g.ld + kB * k + tid] = rd[tid];
}

__global__ void __launch_bounds__(kThreads) k_ldlt_cluster(const double* __restrict__ S, double* ws, int ld, int n,
                                                           double* x, int* solve_ok, Geo g) {
  extern __shared__ double sm[];
  cg::cluster_group cl = cg::this_cluster();
  const int r = (int)cl.block_rank();
  const int C = g.C, nblk = g.nblk;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int rr = tid >> 4, cc = tid & 15;
  __shared__ double s_x[kB];
  __shared__ int s_mine[kMaxBlk + 2];  // panel tiles of this CTA, count last
  double* stW = sm + g.o_stw();
  double* stL = sm + g.o_stl();
  double* Lkk = sm + g.o_lkk();
  double* Td = sm + g.o_diag();

  // copy the lower triangle of S (rows n..ld-1 are the identity) and b into
  // the workspace, tiles dealt round robin; tile (0, 0) goes straight to
  // D(0), which factors it and publishes the factor in its place
  const int nT0 = nblk * (nblk + 1) / 2;
  for (int t0 = r; t0 < nT0 + nblk; t0 += 8 * C) {
    // eight tiles per round: eight loads in flight per thread
    double v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int t = t0 + u * C;
      v[u] = 0.0;
      if (t < nT0) {
        const int i = tri_row(t), j = t - i * (i + 1) / 2;
        v[u] = S[(size_t)(kB * i + rr) * ld + kB * j + cc];
      } else if (t < nT0 + nblk && rr == 0) {
        v[u] = S[(size_t)ld * ld + kB * (t - nT0) + cc];
      }
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int t = t0 + u * C;
      if (t == 0 || t >= nT0 + nblk) continue;
      if (t < nT0) {
        const int i = tri_row(t), j = t - i * (i + 1) / 2;
        ws_lower(ws, ld, i, j)[(size_t)rr * ld + cc] = v[u];
      } else if (rr == 0) {
        ws[(size_t)ld * ld + kB * (t - nT0) + cc] = v[u];
      }
    }
  }
  if (g.diag_cta(0) == r) {
    Td[tid] = S[(size_t)rr * ld + cc];
    __syncthreads();
    factor_publish(g, ws, Td, 0, solve_ok);
  }
  cl.sync();

  for (int k = 0; k < nblk; ++k) {
    // ---- panel.  Tile (k+1, k) goes to D(k+1), which keeps W and L of it in
    //      shared memory for its diagonal update and prefetches tile
    //      (k+1, k+1); the other panel tiles are spread over the other CTAs
    const int Dn = (k + 1 < nblk) ? g.diag_cta(k + 1) : -1;
    if (tid == 0) {
      // this CTA's panel tiles in increasing i (the right-hand side last)
      int nm = 0;
      for (int i = k + 1; i <= nblk; ++i) {
        int x;
        if (i == k + 1 && Dn >= 0) {
          x = Dn;
        } else {
          x = (i - k - 2 + C) % (C - 1);
          if (Dn >= 0 && x >= Dn) ++x;
        }
        if (x == r) s_mine[nm++] = i;
      }
      s_mine[kMaxBlk + 1] = nm;
    }
    double a_diag = 0.0;
    if (r == Dn) a_diag = __ldcg(ws_lower(ws, ld, k + 1, k + 1) + (size_t)rr * ld + cc);
    __syncthreads();
    const int mine = s_mine[kMaxBlk + 1];
    if (mine) {
      Lkk[rr * kPad + cc] = __ldcg(ws_lower(ws, ld, k, k) + (size_t)rr * ld + cc);
      if (tid < kB) Lkk[kPadTile + tid] = __ldcg(ws + (size_t)(ld + 1) * ld + kB * k + tid);
      __syncthreads();
      // work items (panel tile, row pair); warp w takes items w, w + 8, ...
      for (int item = warp; item < mine * (kB / 2); item += 8) {
        const int i = s_mine[item >> 3], p = item & 7;
        if (i == nblk && p > 0) continue;
        const int row = 2 * p + (lane >> 4), c = lane & 15;
        double a = (i < nblk || row == 0) ? __ldcg(ws_tile(ws, ld, nblk, i, k, row, c)) : 0.0;
#pragma unroll
        for (int q = 0; q < kB - 1; ++q) {
          const double wq = __shfl_sync(0xffffffffu, a, (lane & 16) | q);
          if (c > q) a = fma(-wq, Lkk[c * kPad + q], a);
        }
        const double l = a * Lkk[kPadTile + c];
        if (i < nblk) {
          ws_lower(ws, ld, i, k)[(size_t)row * ld + c] = a;
          ws_upper(ws, ld, i, k)[(size_t)row * ld + c] = l;
          if (i == k + 1 && r == Dn) {
            stW[(size_t)i * kTile + row * kB + c] = a;
            stL[(size_t)i * kPadTile + row * kPad + c] = l;
          }
        } else if (row == 0) {
          ws[(size_t)ld * ld + kB * k + c] = a;
          ws[(size_t)(ld + 2) * ld + kB * k + c] = l;
        }
      }
    }
    cl.sync();
    if (k == nblk - 1) break;

    // ---- trailing update of step k; D updates and factors tile (k+1, k+1)
    //      first, then takes its (reduced) range
    const Need nd = trail_need(g, k, r);
    if (r == Dn) {
      // W_{k+1,k} and L_{k+1,k} are already in this CTA's staging area
      const double* wr = stW + (size_t)(k + 1) * kTile + rr * kB;
      const double* lc = stL + (size_t)(k + 1) * kPadTile + cc * kPad;
      double s0 = 0.0, s1 = 0.0;
#pragma unroll
      for (int q = 0; q < kB; q += 2) {
        s0 = fma(wr[q], lc[q], s0);
        s1 = fma(wr[q + 1], lc[q + 1], s1);
      }
      Td[tid] = a_diag - (s0 + s1);
      __syncthreads();
      factor_publish(g, ws, Td, k + 1, solve_ok);
      __syncthreads();
    }
    if (nd.hi > nd.lo) {
      stage_panel(g, ws, k, nd.rmin, nd.rmax, nd.cmin, nd.cmax, stW, stL);
      __syncthreads();
      for (int L0 = nd.lo; L0 < nd.hi; L0 += 8) {
        double av[8];
        int ti[8], tj[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          av[u] = 0.0;
          ti[u] = -1;
          const int L = L0 + u;
          if (L < nd.hi) {
            trail_ij(g, k, L, ti[u], tj[u]);
            if ((ti[u] < nblk || rr == 0) && !(ti[u] == tj[u] && rr < cc))
              av[u] = __ldcg(ws_tile(ws, ld, nblk, ti[u], tj[u], rr, cc));
          }
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          // right-hand-side tiles have only row 0; diagonal tiles are read
          // only on and below the diagonal
          if (ti[u] < 0 || (ti[u] == nblk && rr != 0) || (ti[u] == tj[u] && rr < cc)) continue;
          const double* wr = stW + (size_t)ti[u] * kTile + rr * kB;
          const double* lc = stL + (size_t)tj[u] * kPadTile + cc * kPad;
          double s0 = 0.0, s1 = 0.0;
#pragma unroll
          for (int q = 0; q < kB; q += 2) {
            s0 = fma(wr[q], lc[q], s0);
            s1 = fma(wr[q + 1], lc[q + 1], s1);
          }
          __stcg(ws_tile(ws, ld, nblk, ti[u], tj[u], rr, cc), av[u] - (s0 + s1));
        }
      }
    }
    cl.sync();
  }

  // ---- backward solve L^T x = y on CTA 0 from the workspace; block row
  //      J-1 of L is staged while row J is worked on
  if (r != 0) return;
  if (!*(volatile int*)solve_ok) return;
  double* t = sm + g.o_t();
  double* buf[2] = {sm + g.o_buf(), sm + g.o_buf() + (size_t)nblk * kTile};
  for (int e = tid; e < kB * nblk; e += kThreads) t[e] = __ldcg(ws + (size_t)(ld + 2) * ld + e);
  // block row J of L: L_JJ (strict lower, diagonal tile) and L_JI, I < J;
  // threads [t0, 256) copy it
  auto stage_row = [&](int J, double* dst, int t0) {
    const int step = kThreads - t0, n = (J + 1) * kTile;
    for (int e0 = tid - t0; e0 < n; e0 += 8 * step) {
      double v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int e = e0 + u * step;
        v[u] = 0.0;
        if (e < n) {
          const int I = e >> 8, q = e & 255;
          const double* src = (I == J) ? ws_lower(ws, ld, J, J) : ws_upper(ws, ld, J, I);
          v[u] = __ldcg(src + (size_t)(q >> 4) * ld + (q & 15));
        }
      }
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (e0 + u * step < n) dst[e0 + u * step] = v[u];
    }
  };
  stage_row(nblk - 1, buf[(nblk - 1) & 1], 0);
  __syncthreads();
  for (int J = nblk - 1; J >= 0; --J) {
    const double* Lr = buf[J & 1];
    if (warp == 0) {
      // x_J: unit upper solve L_JJ^T x_J = t_J
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
    } else if (J >= 1) {
      stage_row(J - 1, buf[(J - 1) & 1], 32);  // meanwhile the other warps stage row J-1
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
    __syncthreads();
  }
}

Geo make_geo(int C, int ld, int n) {
  Geo g{};
  g.C = C;
  g.nblk = (n + kB - 1) / kB;
  g.ld = ld;
  g.n = n;
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

cudaError_t chol_cluster_launch(const CholPlan& plan, const double* S, double* ws, int ld, int n, double* x,
                                int* solve_ok, cudaStream_t st) {
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
  return cudaLaunchKernelEx(&cfg, k_ldlt_cluster, S, ws, ld, n, x, solve_ok, g);
}

}  // namespace mcba
