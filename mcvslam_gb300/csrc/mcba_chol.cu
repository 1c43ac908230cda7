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
// Cost model on GB300 (measured): a dependent FP64 FMA takes 64 cycles, one
// FP64 warp instruction occupies its SM sub-partition for 64 cycles (about 2
// FMA per clock per SM), and an FP64 reciprocal with its Newton step takes
// ~240 cycles.  A 16-pivot diagonal tile therefore costs thousands of cycles
// of pure dependency chain, while the trailing updates are FP64-throughput
// work that one SM cannot absorb.  The kernel splits the two:
//
//   * CTA 0 (the chain CTA) runs the critical path and nothing else: for
//     k = 0, 1, ...: factor diagonal tile k (pivot chain on warp 0, pivot
//     application on other warps), solve panel tile (k+1, k) against it and
//     apply step k to diagonal tile (k+1, k+1), which it keeps in shared
//     memory for the next factorisation.  Its ninth warp publishes each
//     result to an L2-resident workspace and prefetches the two tiles the
//     next step needs; the arithmetic warps hand results to it through
//     arrive/sync barriers and never wait for its stores or fences.
//   * CTAs 1..C-1 (workers) run every other task in one fixed global order,
//     dealt round robin: panel solves (i, k) for i >= k+2 and the right-hand
//     side, the trailing updates A_ij -= W_ik L_jk^T, and the inverses
//     M_J = L_JJ^-T for the backward solve.  The order is the right-looking
//     schedule with lookahead: per step k, the panels, then the updates of
//     block columns k+1 and k+2, then the deferred bulk of step k-1, then
//     block column k+3 of step k, then the inverse of diagonal tile k-1.
//     Every task's inputs come earlier in that order (or from the chain
//     CTA's step k), so waiting on them in order cannot deadlock.  A
//     worker's ninth warp stores each result, fences it and releases its
//     flag while the arithmetic warps go on with the next task.
//   * The workspace is tile-major: 16x16 tiles of 2 KB, lower positions for
//     the working tiles (A, then W = L D after its panel solve), upper
//     positions (j, i) for L_ij.  Each tile has a version flag: the number of
//     trailing updates applied (0..j), and j+1 once its panel is solved (for
//     a diagonal tile, once it is factored).  A producer stores, fences and
//     releases the flag; a consumer acquires it (bounded wait) and reads the
//     tile from L2.  Version 0 of every tile is S itself.
//   * Backward solve L^T x = y on the chain CTA, block row by block row:
//     rows of L and M arrive in shared memory by bulk asynchronous copies
//     (one per tile), and per block row only two 16x16 products lie on the
//     dependency chain (u = t_J - L_{J+1,J}^T x_{J+1}, x_J = M_J u).
//
// Every wait has an iteration limit; a CTA that runs out sets an abort word
// that ends all other waits at once, and the solve then reports failure
// (*solve_ok = 0) instead of hanging.  A pivot <= 0 clears *solve_ok; the
// chain CTA, which factors every diagonal tile, then leaves x untouched.  No
// CTA reads another CTA's shared memory.

#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "mcba_chol.h"

namespace mcba {
namespace {

namespace cg = cooperative_groups;

constexpr int kB = 16;         // tile edge
constexpr int kThreads = 288;  // warps 0-7: tile arithmetic; warp 8: copies, fences and flags
constexpr int kMath = 256;
constexpr int kTile = kB * kB;
constexpr int kPad = kB + 1;  // row stride of staged tiles (conflict-free column reads)
constexpr int kPadTile = kB * kPad;
constexpr int kMaxBlk = 24;                // block rows handled by the cluster solve (n <= 384)
constexpr unsigned kSpinLimit = 1u << 21;  // polls per wait (~1 s) before the solve gives up

// named barriers (0 is __syncthreads)
constexpr int kBarPivot = 1;    // pivot chain and pivot application (160 threads)
constexpr int kBarMath = 2;     // warps 0-7
constexpr int kBarPanel = 3;    // chain CTA: panel result ready for warp 8 (288)
constexpr int kBarOutFull = 4;  // workers: result buffer b ready for warp 8 (288), ids 4, 5
constexpr int kBarOutFree = 6;  // workers: result buffer b stored (288), ids 6, 7

// Reciprocal of a pivot: rcp.approx.ftz.f64 (relative error ~1e-6), then one
// cubic Newton-Raphson step y (1 + e + e^2), e = 1 - d y, which leaves an
// error far below FP64 round-off.  Pivots whose reciprocal would leave the
// normal range take the IEEE division (integer test on the exponent field,
// evaluated beside the approximation).
__device__ __forceinline__ double recip_pivot(double d) {
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(d));
  const unsigned ex = ((unsigned)(__double_as_longlong(d) >> 52)) & 0x7ffu;
  if (ex < 0x040u || ex > 0x7bfu) return 1.0 / d;
  const double e = fma(-d, y, 1.0);
  const double p = fma(e, e, e);
  return fma(y, p, y);
}

__device__ __forceinline__ void bar_sync(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

__device__ __forceinline__ void bar_arrive(int id, int nthreads) {
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async;" ::: "memory"); }

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// Bulk asynchronous copy global -> this CTA's shared memory, completion
// counted in bytes on the mbarrier (addresses 16-byte aligned, size a
// multiple of 16).
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for *p >= v (one thread).  Returns false when this wait ran
// out (it then sets the abort word) or another CTA already gave up.
__device__ bool wait_ge(const int* p, int v, int* abort_word) {
  for (unsigned it = 0; it < kSpinLimit; ++it) {
    if (ld_acquire(p) >= v) return true;
    if ((it & 63u) == 0 && ld_acquire(abort_word) != 0) return false;
    if (it > 32) __nanosleep(64);
  }
  atomicExch(abort_word, 1);
  return false;
}

// Bounded wait for an mbarrier phase; gives up like wait_ge.
__device__ void mbar_wait(uint64_t* bar, unsigned parity, int* abort_word) {
  for (unsigned it = 0; it < kSpinLimit; ++it) {
    if (mbar_try_wait(bar, parity)) return;
    if ((it & 63u) == 0 && ld_acquire(abort_word) != 0) return;
  }
  atomicExch(abort_word, 1);
}

struct Geo {
  int C, nblk, ld, n, R;  // R: backward-solve row slots in shared memory
  // workspace (doubles): nblk x nblk tiles of 256, then the right-hand-side
  // rows W, 1/d and y (16 nblk each), then (as ints) the version flags
  // ((nblk + 1) x nblk), one flag per inverse M_J and the abort word, then
  // the inverses M_J (256 each, transposed), each part 256-byte aligned
  __host__ __device__ size_t tile_off(int i, int j) const { return ((size_t)i * nblk + j) * kTile; }
  __host__ __device__ size_t rhs_w() const { return (size_t)nblk * nblk * kTile; }
  __host__ __device__ size_t rhs_rd() const { return rhs_w() + (size_t)kB * nblk; }
  __host__ __device__ size_t rhs_y() const { return rhs_rd() + (size_t)kB * nblk; }
  __host__ __device__ size_t flag_offset() const { return ((rhs_y() + (size_t)kB * nblk + 31) / 32) * 32; }
  __host__ __device__ int inv_index(int J) const { return (nblk + 1) * nblk + J; }
  __host__ __device__ int abort_index() const { return (nblk + 2) * nblk; }
  __host__ __device__ int flag_count() const { return (nblk + 2) * nblk + 1; }
  __host__ __device__ size_t m_offset() const { return flag_offset() + (((size_t)flag_count() + 63) / 64) * 32; }
  __host__ __device__ size_t ws_doubles() const { return m_offset() + (size_t)nblk * kTile; }
  // chain CTA shared memory (doubles): two diagonal tiles with 1/d and the
  // squares of the sub-diagonal, the incoming panel tile, W and L of the
  // panel, the padded copy of L_kk with 1/d
  __host__ __device__ size_t c_diag(int b) const { return (size_t)b * (kTile + 2 * kB); }
  __host__ __device__ size_t c_p() const { return 2 * (size_t)(kTile + 2 * kB); }
  __host__ __device__ size_t c_wp() const { return c_p() + kTile; }
  __host__ __device__ size_t c_lp() const { return c_wp() + kPadTile; }
  __host__ __device__ size_t c_lk() const { return c_lp() + kPadTile; }
  __host__ __device__ size_t c_end() const { return c_lk() + kPadTile + kB; }
  // backward solve, after that: t, x, the slot mbarriers, R row slots
  __host__ __device__ size_t b_t() const { return c_end(); }
  __host__ __device__ size_t b_x() const { return b_t() + (size_t)kB * nblk; }
  __host__ __device__ size_t b_bar() const { return b_x() + (size_t)kB * nblk; }
  __host__ __device__ size_t b_slot(int s) const { return b_bar() + (size_t)((R + 1) & ~1) + (size_t)s * nblk * kTile; }
  __host__ __device__ size_t b_end() const { return b_slot(R); }
  // worker: staged W and L tiles, the padded L_kk with 1/d, two result
  // buffers of 512
  __host__ __device__ size_t w_w() const { return 0; }
  __host__ __device__ size_t w_l() const { return kPadTile; }
  __host__ __device__ size_t w_lk() const { return 2 * kPadTile; }
  __host__ __device__ size_t w_out(int b) const { return 3 * kPadTile + kB + (size_t)b * 2 * kTile; }
  __host__ __device__ size_t w_end() const { return w_out(2); }
  __host__ __device__ size_t total() const {
    size_t t = c_end();
    if (b_end() > t) t = b_end();
    if (w_end() > t) t = w_end();
    return t;
  }
};

// Element (rr, cc) of tile (i, j) of S (row stride ld; block row nblk is the
// right-hand side, row ld, where only rr = 0 exists).
__device__ __forceinline__ size_t s_at(int ld, int nblk, int i, int j, int rr, int cc) {
  return (i < nblk) ? (size_t)(kB * i + rr) * ld + kB * j + cc : (size_t)ld * ld + kB * j + cc;
}
// The same element in the workspace.
__device__ __forceinline__ size_t w_at(const Geo& g, int i, int j, int rr, int cc) {
  return (i < g.nblk) ? g.tile_off(i, j) + rr * kB + cc : g.rhs_w() + kB * j + cc;
}
// L_ij (i > j) in the workspace: the upper tile position (j, i).
__device__ __forceinline__ size_t l_at(const Geo& g, int i, int j, int rr, int cc) {
  return g.tile_off(j, i) + rr * kB + cc;
}
__device__ __forceinline__ int* flag_at(int* fl, int nblk, int i, int j) { return fl + i * nblk + j; }

// Version v of a tile element: S for v = 0, the workspace after that.
__device__ __forceinline__ double tile_read(const Geo& g, const double* S, const double* ws, int i, int j, int rr,
                                            int cc, int v) {
  return v == 0 ? S[s_at(g.ld, g.nblk, i, j, rr, cc)] : __ldcg(ws + w_at(g, i, j, rr, cc));
}

// Wait of the arithmetic warps on up to three flags, one spinning thread per
// warp 0..2, then a barrier of warps 0-7.
__device__ void math_wait3(int* f0, int v0, int* f1, int v1, int* f2, int v2, int* abort_word) {
  const int tid = threadIdx.x;
  if (tid == 0 && f0) wait_ge(f0, v0, abort_word);
  if (tid == 32 && f1) wait_ge(f1, v1, abort_word);
  if (tid == 64 && f2) wait_ge(f2, v2, abort_word);
  bar_sync(kBarMath, kMath);
}

// Forward substitution of two rows per warp against a unit lower L (padded
// copy Lk): a_row <- a_row L^-T.  Lanes 0-15 hold row 2w, lanes 16-31 row
// 2w+1; the result is W (multiply by 1/d for L).
__device__ __forceinline__ double fwd_rows(double a, const double* Lk, int lane) {
  const int c = lane & 15;
#pragma unroll
  for (int q = 0; q < kB - 1; ++q) {
    const double wq = __shfl_sync(0xffffffffu, a, (lane & 16) | q);
    if (c > q) a = fma(-wq, Lk[c * kPad + q], a);
  }
  return a;
}

// L D L^T of one 16x16 diagonal tile in place: strict lower part <- L,
// diagonal <- d, rd <- 1/d.  The pivot chain runs alone on warp 0 (its own
// sub-partition, so no other FP64 work queues in front of it): from r_j it
// forms d_{j+1} = a_{j+1,j+1} - a_{j+1,j}^2 r_j itself and takes its
// reciprocal, while warps 1-3 and 5 apply pivot j to the other entries.
// Entry (i, m), 1 <= m <= i, sits on update thread u in order of decreasing
// column, so the entries still active at pivot j are the first
// (15-j)(16-j)/2 threads and whole warps fall idle early (warp 5, which
// shares warp 1's sub-partition, after pivot 1).  The diagonal entry skips
// the pivot that warp 0 applies, and entry (i, i-1) leaves its square in
// sq[i] once final.  One named barrier per pivot; warps 4 and 6-8 take no
// part.  The arithmetic is the plain right-looking LDL^T.
__device__ void diag_ldlt(double* T, double* rd, double* sq, int* solve_ok) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  constexpr int kPart = 160;  // warps 0-3 and 5
  if (warp == 0) {
    double r = recip_pivot(T[0]);
    if (lane == 0) rd[0] = r;
    for (int j = 0; j < kB; ++j) {
      bar_sync(kBarPivot, kPart);  // pivot j-1 applied everywhere, r_j published
      if (j + 1 < kB) {
        const double s = (j == 0) ? T[kB] * T[kB] : sq[j + 1];
        const double d = fma(-s, r, T[(j + 1) * kB + j + 1]);
        if (lane == 0) T[(j + 1) * kB + j + 1] = d;
        r = recip_pivot(d);
        if (lane == 0) rd[j + 1] = r;
      }
    }
    bar_sync(kBarPivot, kPart);
    if (lane < kB && !(T[lane * kB + lane] > 0.0)) *solve_ok = 0;
  } else {
    const int u = (warp < 4) ? (warp - 1) * 32 + lane : 96 + lane;
    const bool has = u < 120;
    int um = 15, rem = has ? u : 0;
    while (rem >= kB - um) {
      rem -= kB - um;
      --um;
    }
    const int ui = um + rem;
    double* Tu = T + ui * kB + um;
    for (int j = 0; j < kB; ++j) {
      bar_sync(kBarPivot, kPart);
      if (has && um > j && !(ui == um && um == j + 1)) {
        const double prod = T[ui * kB + j] * T[um * kB + j];
        const double v = fma(-prod, rd[j], *Tu);
        *Tu = v;
        if (um == ui - 1 && j == um - 1) sq[ui] = v * v;
      }
    }
    bar_sync(kBarPivot, kPart);
    if (has) T[ui * kB + (um - 1)] *= rd[um - 1];
  }
}

// One backward-solve row J into a shared-memory slot by bulk asynchronous
// copies, one per tile: L_JI (I < J) into positions I, M_J into position J
// (unless the chain CTA computed it in place).  Run by one whole warp once
// every producer is known to be done.
__device__ void issue_row(const Geo& g, const double* ws, double* slot, uint64_t* bar, int J, bool with_m) {
  const int lane = threadIdx.x & 31;
  const int ncopy = J + (with_m ? 1 : 0);
  if (lane == 0) mbar_expect_tx(bar, (unsigned)ncopy * kTile * sizeof(double));
  __syncwarp();
  for (int I = lane; I < ncopy; I += 32) {
    const double* src = (I < J) ? ws + g.tile_off(I, J) : ws + g.m_offset() + (size_t)J * kTile;
    bulk_g2s(slot + I * kTile, src, kTile * sizeof(double), bar);
  }
}

// ------------------------------------------------------------ chain CTA --

__device__ void chain_cta(const Geo& g, const double* __restrict__ S, double* ws, double* x, int* solve_ok, int* fl,
                          double* sm) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int rr = (tid >> 4) & 15, cc = tid & 15;
  const int nblk = g.nblk, ld = g.ld, R = g.R;
  int* abort_word = fl + g.abort_index();
  double* const Tb0 = sm + g.c_diag(0);
  double* const Tb1 = sm + g.c_diag(1);
  double* P = sm + g.c_p();
  double* Wp = sm + g.c_wp();
  double* Lp = sm + g.c_lp();
  double* Lk = sm + g.c_lk();
  double* t = sm + g.b_t();
  double* xs = sm + g.b_x();
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + g.b_bar());
  auto slot = [&](int J) { return sm + g.b_slot(J % R); };
  int cur = 0;
  if (tid < kMath) Tb0[tid] = S[(size_t)rr * ld + cc];
  if (tid == kMath) {
    for (int b = 0; b < R; ++b) mbar_init(bars + b, 1);
    fence_mbar_init();
  }
  __syncthreads();

  for (int k = 0; k + 1 < nblk; ++k) {
    double* T = cur ? Tb1 : Tb0;
    double* Q = cur ? Tb0 : Tb1;
    // ---- (a) factor diagonal tile k; warp 8 fetches tiles (k+1, k) and
    //      (k+1, k+1) at version k meanwhile
    if (warp < 8) {
      if (warp < 4 || warp == 5) diag_ldlt(T, T + kTile, T + kTile + kB, solve_ok);
    } else {
      if (k > 0) {
        if (lane == 0) wait_ge(flag_at(fl, nblk, k + 1, k), k, abort_word);
        if (lane == 1) wait_ge(flag_at(fl, nblk, k + 1, k + 1), k, abort_word);
        __syncwarp();
      }
      double v[16];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int e = lane + 32 * u;
        v[u] = tile_read(g, S, ws, k + 1, k, e >> 4, e & 15, k);
        v[8 + u] = tile_read(g, S, ws, k + 1, k + 1, e >> 4, e & 15, k);
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        P[lane + 32 * u] = v[u];
        Q[lane + 32 * u] = v[8 + u];
      }
    }
    __syncthreads();

    // ---- (b) warps 0-7 solve panel tile (k+1, k): W = A L_kk^-T (row by
    //      row), L = W D_k^-1, and hand it to warp 8; warp 8 publishes L_kk,
    //      d and 1/d, then W and L of the panel
    if (warp < 8) {
      Lk[rr * kPad + cc] = T[tid];
      if (tid < kB) Lk[kPadTile + tid] = T[kTile + tid];
      bar_sync(kBarMath, kMath);
      const int row = 2 * warp + (lane >> 4), c = lane & 15;
      const double a = fwd_rows(P[row * kB + c], Lk, lane);
      Wp[row * kPad + c] = a;
      Lp[row * kPad + c] = a * Lk[kPadTile + c];
      bar_arrive(kBarPanel, kThreads);
      bar_sync(kBarMath, kMath);  // (c) reads rows of W and L written by other warps
    } else {
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int e = lane + 32 * u;
        if ((e >> 4) >= (e & 15)) __stcg(ws + g.tile_off(k, k) + e, T[e]);
      }
      if (lane < kB) __stcg(ws + g.rhs_rd() + kB * k + lane, T[kTile + lane]);
      __threadfence();
      __syncwarp();
      if (lane == 0) st_release(flag_at(fl, nblk, k, k), k + 1);
      bar_sync(kBarPanel, kThreads);
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int e = lane + 32 * u, r0 = e >> 4, c0 = e & 15;
        __stcg(ws + g.tile_off(k + 1, k) + e, Wp[r0 * kPad + c0]);
        __stcg(ws + g.tile_off(k, k + 1) + e, Lp[r0 * kPad + c0]);
      }
      __threadfence();
      __syncwarp();
      if (lane == 0) st_release(flag_at(fl, nblk, k + 1, k), k + 1);
    }
    // ---- (c) warps 0-7 apply step k to diagonal tile (k+1, k+1) (lower part)
    if (warp < 8 && rr >= cc) {
      const double* wr = Wp + rr * kPad;
      const double* lc = Lp + cc * kPad;
      double s0 = 0.0, s1 = 0.0;
#pragma unroll
      for (int q = 0; q < kB; q += 2) {
        s0 = fma(wr[q], lc[q], s0);
        s1 = fma(wr[q + 1], lc[q + 1], s1);
      }
      Q[tid] -= s0 + s1;
    }
    if (warp < 8) bar_sync(kBarMath, kMath);
    cur ^= 1;
  }

  // ---- last diagonal tile: factor it; warp 8 fetches the last
  //      right-hand-side tile meanwhile.  Then M = L^-T of the tile goes
  //      straight into its backward-solve slot and the last y into t.
  {
    const int k = nblk - 1;
    double* T = cur ? Tb1 : Tb0;
    if (warp < 8) {
      if (warp < 4 || warp == 5) diag_ldlt(T, T + kTile, T + kTile + kB, solve_ok);
    } else {
      if (k > 0 && lane == 0) wait_ge(flag_at(fl, nblk, nblk, k), k, abort_word);
      __syncwarp();
      if (lane < kB) P[lane] = tile_read(g, S, ws, nblk, k, 0, lane, k);
    }
    __syncthreads();
    if (tid < kMath) {
      Lk[rr * kPad + cc] = T[tid];
      if (tid < kB) Lk[kPadTile + tid] = T[kTile + tid];
    }
    __syncthreads();
    if (warp < 8) {
      const int row = 2 * warp + (lane >> 4), c = lane & 15;
      const double m = fwd_rows(row == c ? 1.0 : 0.0, Lk, lane);
      slot(k)[k * kTile + c * kB + row] = m;  // M_k stored transposed
    } else {
      const double a = fwd_rows(lane < kB ? P[lane] : 0.0, Lk, lane);
      if (lane < kB) t[kB * k + lane] = a * Lk[kPadTile + lane];
    }
  }

  // ---- backward solve L^T x = y, block row by block row.  Rows reach
  //      shared memory by bulk copies, R slots deep; per row J:
  //        warp 0:     u = t_J - L_{J+1,J}^T x_{J+1};  x_J = M_J u
  //        warps 1-3, 5-7:  t_I -= L_{J+1,I}^T x_{J+1}, I <= J-1
  //        warp 8:     issues row J+2-R
  //      so only the two 16x16 products of warp 0 lie on the chain.
  //      Right-hand-side panel J is done only after every L_JI was (its
  //      updates read them), and the last right-hand-side tile waited above
  //      covers row nblk-1; so warp 8 waits for the right-hand-side panels
  //      and the inverses, one lane per row, then issues rows.
  if (warp == 8) {
    if (lane < nblk - 1) {
      wait_ge(flag_at(fl, nblk, nblk, lane), lane + 1, abort_word);
      wait_ge(fl + g.inv_index(lane), 1, abort_word);
    }
    __syncwarp();
    fence_proxy_async();
    for (int J = nblk - 1; J >= 0 && J >= nblk - R; --J) issue_row(g, ws, slot(J), bars + J % R, J, J < nblk - 1);
  }
  __syncthreads();
  for (int e = tid; e < kB * (nblk - 1); e += kThreads) t[e] = __ldcg(ws + g.rhs_y() + e);
  __syncthreads();
  auto parity = [&](int J) { return (unsigned)(((nblk - 1 - J) / R) & 1); };
  const bool write_x = *(volatile int*)solve_ok != 0;  // every pivot is known by now
  for (int J = nblk - 1; J >= 0; --J) {
    const double* rowJ = slot(J);
    const double* rowJ1 = slot(J + 1);
    if (warp == 0) {
      mbar_wait(bars + J % R, parity(J), abort_word);
      const int h = lane >> 4, c = lane & 15;
      double s = 0.0;
      if (J + 1 < nblk) {
        const double* Lt = rowJ1 + J * kTile;
        const double* xj = xs + kB * (J + 1);
        double p0 = 0.0, p1 = 0.0;
#pragma unroll
        for (int q = 0; q < 8; q += 2) {
          p0 = fma(Lt[(8 * h + q) * kB + c], xj[8 * h + q], p0);
          p1 = fma(Lt[(8 * h + q + 1) * kB + c], xj[8 * h + q + 1], p1);
        }
        s = p0 + p1;
        s += __shfl_xor_sync(0xffffffffu, s, 16);
      }
      const double u = t[kB * J + c] - s;
      const double* Ms = rowJ + J * kTile;
      double p0 = 0.0, p1 = 0.0;
#pragma unroll
      for (int q = 0; q < 8; q += 2) {
        const double u0 = __shfl_sync(0xffffffffu, u, 8 * h + q);
        const double u1 = __shfl_sync(0xffffffffu, u, 8 * h + q + 1);
        p0 = fma(Ms[(8 * h + q) * kB + c], u0, p0);
        p1 = fma(Ms[(8 * h + q + 1) * kB + c], u1, p1);
      }
      double xv = p0 + p1;
      xv += __shfl_xor_sync(0xffffffffu, xv, 16);
      if (lane < kB) {
        xs[kB * J + c] = xv;
        if (kB * J + c < g.n && write_x) x[kB * J + c] = xv;
      }
    } else if (warp < 8 && warp != 4) {
      // warp 4 shares warp 0's sub-partition and stays out of the FP64 work
      if (J + 1 < nblk) {
        const double* xj = xs + kB * (J + 1);
        for (int it = tid - (warp < 4 ? 32 : 64); it < kB * J; it += kMath - 64) {
          const int I = it >> 4, c = it & 15;
          const double* Tm = rowJ1 + I * kTile;
          double v0 = 0.0, v1 = 0.0;
#pragma unroll
          for (int q = 0; q < kB; q += 2) {
            v0 = fma(Tm[q * kB + c], xj[q], v0);
            v1 = fma(Tm[(q + 1) * kB + c], xj[q + 1], v1);
          }
          t[kB * I + c] -= v0 + v1;
        }
      }
    } else if (warp == 8) {
      const int Jn = J + 2 - R;
      if (Jn >= 0 && Jn < nblk - R) issue_row(g, ws, slot(Jn), bars + Jn % R, Jn, true);
    }
    __syncthreads();
  }
  if (tid == 0 && ld_acquire(abort_word) != 0) *solve_ok = 0;
}

// --------------------------------------------------------------- workers --
//
// Warps 0-7 run each task into result buffer b (tasks alternate between two
// buffers); warp 8 then stores the result, fences it and releases its flag.
// Task kinds and what warp 8 stores:
//   panel (i, k): W to tile (i, k), L to tile (k, i) (the right-hand side:
//                 the W and y rows), flag (i, k) = k+1
//   update (i, j, s): tile (i, j) (lower part of a diagonal tile, row 0 of
//                 the right-hand side), flag (i, j) = s+1
//   inverse J:    M_J, inverse flag J = 1
enum : int { kTaskPanel = 0, kTaskUpdate = 1, kTaskInv = 2 };

__device__ void task_store(const Geo& g, double* ws, int* fl, const double* out, int kind, int i, int j, int s) {
  const int lane = threadIdx.x & 31;
  const int nblk = g.nblk;
  int* f = nullptr;
  int v = 0;
  if (kind == kTaskPanel) {
    if (i < nblk) {
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int e = lane + 32 * u;
        __stcg(ws + g.tile_off(i, j) + e, out[e]);
        __stcg(ws + g.tile_off(j, i) + e, out[kTile + e]);
      }
    } else if (lane < kB) {
      __stcg(ws + g.rhs_w() + kB * j + lane, out[lane]);
      __stcg(ws + g.rhs_y() + kB * j + lane, out[kTile + lane]);
    }
    f = flag_at(fl, nblk, i, j);
    v = j + 1;
  } else if (kind == kTaskUpdate) {
    if (i < nblk) {
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int e = lane + 32 * u;
        if (i != j || (e >> 4) >= (e & 15)) __stcg(ws + g.tile_off(i, j) + e, out[e]);
      }
    } else if (lane < kB) {
      __stcg(ws + g.rhs_w() + kB * j + lane, out[lane]);
    }
    f = flag_at(fl, nblk, i, j);
    v = s + 1;
  } else {
#pragma unroll
    for (int u = 0; u < 8; ++u) __stcg(ws + g.m_offset() + (size_t)i * kTile + lane + 32 * u, out[lane + 32 * u]);
    f = fl + g.inv_index(i);
    v = 1;
  }
  __threadfence();
  __syncwarp();
  if (lane == 0) st_release(f, v);
}

// Panel tile (i, k), i >= k+2 (i = nblk: the right-hand side), at version k:
// W = A L_kk^-T, L = W D_k^-1 into out[0..256) and out[256..512).
__device__ void math_panel(const Geo& g, const double* __restrict__ S, const double* ws, int* fl, double* sm,
                           double* out, int i, int k) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nblk = g.nblk;
  int* abort_word = fl + g.abort_index();
  double* Lk = sm + g.w_lk();
  math_wait3(k > 0 ? flag_at(fl, nblk, i, k) : nullptr, k, flag_at(fl, nblk, k, k), k + 1, nullptr, 0, abort_word);
  const bool rhs = (i == nblk);
  const int row = 2 * warp + (lane >> 4), c = lane & 15;
  double a = 0.0;
  if (!rhs || row == 0) a = tile_read(g, S, ws, i, k, row, c, k);
  Lk[(tid >> 4) * kPad + (tid & 15)] = __ldcg(ws + g.tile_off(k, k) + tid);
  if (tid < kB) Lk[kPadTile + tid] = __ldcg(ws + g.rhs_rd() + kB * k + tid);
  bar_sync(kBarMath, kMath);
  if (!rhs || warp == 0) {
    a = fwd_rows(a, Lk, lane);
    out[row * kB + c] = a;
    out[kTile + row * kB + c] = a * Lk[kPadTile + c];
  }
}

// M_J = L_JJ^-T: the panel solve of the identity, stored transposed
// (M_J[c][q] at [q * 16 + c]).
__device__ void math_inv(const Geo& g, const double* ws, int* fl, double* sm, double* out, int J) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  int* abort_word = fl + g.abort_index();
  double* Lk = sm + g.w_lk();
  math_wait3(flag_at(fl, g.nblk, J, J), J + 1, nullptr, 0, nullptr, 0, abort_word);
  Lk[(tid >> 4) * kPad + (tid & 15)] = __ldcg(ws + g.tile_off(J, J) + tid);
  bar_sync(kBarMath, kMath);
  const int row = 2 * warp + (lane >> 4), c = lane & 15;
  out[c * kB + row] = fwd_rows(row == c ? 1.0 : 0.0, Lk, lane);
}

// Trailing update of tile (i, j) with step s: A_ij -= W_is L_js^T.
__device__ void math_update(const Geo& g, const double* __restrict__ S, const double* ws, int* fl, double* sm,
                            double* out, int i, int j, int s) {
  const int tid = threadIdx.x;
  const int nblk = g.nblk;
  int* abort_word = fl + g.abort_index();
  double* Wt = sm + g.w_w();
  double* Lt = sm + g.w_l();
  math_wait3(s > 0 ? flag_at(fl, nblk, i, j) : nullptr, s, flag_at(fl, nblk, i, s), s + 1, flag_at(fl, nblk, j, s),
             s + 1, abort_word);
  const bool rhs = (i == nblk);
  const int rr = tid >> 4, cc = tid & 15;
  const bool mine = rhs ? rr == 0 : (i != j || rr >= cc);
  double a = 0.0;
  if (mine) a = tile_read(g, S, ws, i, j, rr, cc, s);
  if (!rhs || rr == 0) Wt[rr * kPad + cc] = __ldcg(ws + w_at(g, i, s, rr, cc));
  Lt[rr * kPad + cc] = __ldcg(ws + l_at(g, j, s, rr, cc));
  bar_sync(kBarMath, kMath);
  if (mine) {
    const double* wr = Wt + rr * kPad;
    const double* lc = Lt + cc * kPad;
    double s0 = 0.0, s1 = 0.0;
#pragma unroll
    for (int q = 0; q < kB; q += 2) {
      s0 = fma(wr[q], lc[q], s0);
      s1 = fma(wr[q + 1], lc[q + 1], s1);
    }
    out[tid] = a - (s0 + s1);
  }
}

// The worker's share of a segment of cnt tasks of the global order: task m
// of the order goes to worker m mod W.
struct Deal {
  int W, w, m;
  template <typename F>
  __device__ __forceinline__ void segment(int cnt, F&& f) {
    if (cnt <= 0) return;
    int first = (w - m) % W;
    if (first < 0) first += W;
    for (int idx = first; idx < cnt; idx += W) f(idx);
    m += cnt;
  }
};

// Calls f(kind, i, j, s) for this worker's tasks in order.
template <typename F>
__device__ void worker_tasks(const Geo& g, int rank, F&& f) {
  const int nblk = g.nblk;
  Deal d{g.C - 1, rank - 1, 0};
  for (int k = 0; k < nblk; ++k) {
    // (1) panels (i, k), i >= k+2, right-hand side last (the last column's
    //     right-hand-side panel is the chain CTA's)
    if (k + 1 < nblk) d.segment(nblk - k - 1, [&](int idx) { f(kTaskPanel, k + 2 + idx, k, k); });
    // (2) step k on block column k+1 below its diagonal tile (the chain CTA
    //     updates the diagonal tile itself)
    if (k + 1 < nblk) d.segment(nblk - k - 1, [&](int idx) { f(kTaskUpdate, k + 2 + idx, k + 1, k); });
    // (3) step k on block column k+2, diagonal tile included
    if (k + 2 < nblk) d.segment(nblk - k - 1, [&](int idx) { f(kTaskUpdate, k + 2 + idx, k + 2, k); });
    // (4b) the deferred bulk of step k-1: block columns k+3 .. nblk-1
    if (k >= 1 && k + 3 < nblk) {
      int cnt = 0;
      for (int j = k + 3; j < nblk; ++j) cnt += nblk - j + 1;
      d.segment(cnt, [&](int idx) {
        int j = k + 3;
        while (idx >= nblk - j + 1) {
          idx -= nblk - j + 1;
          ++j;
        }
        f(kTaskUpdate, j + idx, j, k - 1);
      });
    }
    // (4a) step k on block column k+3
    if (k + 3 < nblk) d.segment(nblk - k - 2, [&](int idx) { f(kTaskUpdate, k + 3 + idx, k + 3, k); });
    // (5) the backward-solve inverse of diagonal tile k-1
    if (k >= 1) d.segment(1, [&](int) { f(kTaskInv, k - 1, k - 1, 0); });
  }
}

__device__ void worker_cta(const Geo& g, const double* __restrict__ S, double* ws, int* fl, double* sm, int rank) {
  const int warp = threadIdx.x >> 5;
  int n = 0;  // tasks run so far; result buffer n & 1
  if (warp < 8) {
    worker_tasks(g, rank, [&](int kind, int i, int j, int s) {
      const int b = n & 1;
      double* out = sm + g.w_out(b);
      if (n >= 2) bar_sync(kBarOutFree + b, kThreads);  // warp 8 has stored task n-2
      if (kind == kTaskPanel)
        math_panel(g, S, ws, fl, sm, out, i, j);
      else if (kind == kTaskUpdate)
        math_update(g, S, ws, fl, sm, out, i, j, s);
      else
        math_inv(g, ws, fl, sm, out, i);
      bar_arrive(kBarOutFull + b, kThreads);
      ++n;
    });
    // balance warp 8's last two releases
    for (int q = max(n - 2, 0); q < n; ++q) bar_sync(kBarOutFree + (q & 1), kThreads);
  } else {
    worker_tasks(g, rank, [&](int kind, int i, int j, int s) {
      const int b = n & 1;
      bar_sync(kBarOutFull + b, kThreads);
      task_store(g, ws, fl, sm + g.w_out(b), kind, i, j, s);
      bar_arrive(kBarOutFree + b, kThreads);
      ++n;
    });
  }
}

__global__ void __launch_bounds__(kThreads, 1) k_ldlt_cluster(const double* __restrict__ S, double* ws, double* x,
                                                              int* solve_ok, Geo g) {
  extern __shared__ __align__(16) double sm[];
  cg::cluster_group cl = cg::this_cluster();
  const int r = (int)cl.block_rank();
  int* fl = reinterpret_cast<int*>(ws + g.flag_offset());
  // the version flags and the abort word start at zero in every launch
  for (int e = r * kThreads + (int)threadIdx.x; e < g.flag_count(); e += g.C * kThreads) fl[e] = 0;
  __threadfence();
  cl.sync();
  if (r == 0)
    chain_cta(g, S, ws, x, solve_ok, fl, sm);
  else
    worker_cta(g, S, ws, fl, sm, r);
}

Geo make_geo(int C, int ld, int n, int R) {
  Geo g{};
  g.C = C;
  g.nblk = (n + kB - 1) / kB;
  g.ld = ld;
  g.n = n;
  g.R = R;
  return g;
}

}  // namespace

int chol_cluster_plan(int ld, int n, CholPlan* plan) {
  plan->ok = false;
  const int nblk = (n + kB - 1) / kB;
  if (n <= 0 || ld < kB * nblk || nblk > kMaxBlk) return 0;
  // the tiles, flags and inverses must fit the (ld + 32) x ld workspace
  if (make_geo(16, ld, n, 1).ws_doubles() > (size_t)(ld + 32) * ld) return 0;
  int dev = 0;
  cudaGetDevice(&dev);
  int max_smem = 0;
  cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const int reserve = 1024;  // static shared memory of the kernel
  if (cudaFuncSetAttribute(k_ldlt_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess ||
      cudaFuncSetAttribute(k_ldlt_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem - reserve) !=
          cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  // as many backward-solve row slots as fit (all rows when possible), at
  // least three
  int R = nblk;
  while (R > std::min(nblk, 3) && make_geo(16, ld, n, R).total() * sizeof(double) + reserve > (size_t)max_smem) --R;
  for (int C : {16, 8}) {
    const Geo g = make_geo(C, ld, n, R);
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
    plan->slots = R;
    plan->smem_bytes = bytes;
    return 1;
  }
  return 0;
}

cudaError_t chol_cluster_launch(const CholPlan& plan, const double* S, double* ws, int ld, int n, double* x,
                                int* solve_ok, cudaStream_t st) {
  const Geo g = make_geo(plan.cluster, ld, n, plan.slots);
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
  return cudaLaunchKernelEx(&cfg, k_ldlt_cluster, S, ws, x, solve_ok, g);
}

}  // namespace mcba
