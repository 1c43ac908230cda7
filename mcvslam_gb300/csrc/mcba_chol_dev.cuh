// mcba_chol_dev.cuh -- device side of the FP64 solve of the reduced camera
// system on one thread-block cluster (included by mcba_chol.cu, which
// launches it as its own kernel, and by mcba_solver.cu, whose persistent
// window kernel runs it inside its own clusters).
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
//     dealt round robin: panel solves (i, k) for i >= k+3 and the right-hand
//     side, and the trailing updates A_ij -= W_ik L_jk^T.  The order is the right-looking
//     schedule with lookahead: per step k, the panels, then the updates of
//     block columns k+1 and k+2, then the deferred bulk of step k-1, then
//     block column k+3 of step k.
//     Every task's inputs come earlier in that order (or from the chain
//     CTA's step k), so waiting on them in order cannot deadlock.  A
//     worker's warps 8 and 9 store each result (fence, flag) and stage the
//     next task's inputs while warps 0-7 compute.
//   * Worker 1 runs only block row k+2 of each step k: its panel, then the
//     updates of its tiles (k+2, k+1) and (k+2, k+2), which it pushes
//     straight into the chain CTA's shared memory (st.async, counted on an
//     mbarrier there) as the chain CTA's inputs for step k+1; then the
//     inverse M_k of diagonal tile k.
//   * The workspace is tile-major: 16x16 tiles of 2 KB, lower positions for
//     the working tiles (A, then W = L D after its panel solve), upper
//     positions (j, i) for L_ij.  Each tile has a version flag: the number of
//     trailing updates applied (0..j), and j+1 once its panel is solved (for
//     a diagonal tile, once it is factored).  A producer stores the tile,
//     fences and releases the flag; a consumer acquires it (bounded wait)
//     and reads the tile from L2.  Version 0 of every tile is S itself.  The
//     flags live in the chain CTA's shared memory and every CTA reaches them
//     through the cluster's distributed shared memory (release/acquire at
//     cluster scope): in global memory their polls took the L2 round trip of
//     whichever die the flag's line maps to, and the factorisation time
//     depended on that (98 or 104 us at n = 168 on GB300, by the page).
//   * Backward solve L^T x = y on the chain CTA, block row by block row:
//     per block row only one 16x16 product lies on the dependency chain
//     (x_J = M_J t_J - P_J x_{J+1}, with P_J = M_J L_{J+1,J}^T formed beside
//     M_J by the lookahead worker and M_J t_J by a second warp); six helper
//     warps apply the other terms of t as the rows of x appear, handing over
//     through counters in shared memory, and every warp loads its tiles
//     from L2 into registers two uses ahead.
//
// Every wait has a time limit (%globaltimer); a wait that runs out sets an
// abort word, and the solve then reports failure (*solve_ok = 0) instead of
// hanging.  Waits on the workers' flags end at once when the abort word is
// set.  The waits that guard shared memory (the pushes into the chain CTA
// and the lookahead worker's wait for the chain CTA's panel, which orders
// its pushes after the chain CTA's mbarrier arms) run to completion even
// then, as do the chain CTA's waits on its own warps: their producers run
// whatever
// the other flags say, so no copy into shared memory is in flight when a CTA
// leaves.  A pivot <= 0 clears *solve_ok; the
// chain CTA, which factors every diagonal tile, then leaves x untouched.
// Apart from the flags (and the abort word beside them), no CTA reads
// another CTA's shared memory; a cluster barrier at the end keeps the chain
// CTA, which holds them, until every CTA is done with them.


#pragma once

#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace mcba {
namespace chold {
namespace {

namespace cg = cooperative_groups;

constexpr int kB = 16;         // tile edge
constexpr int kThreads = 320;  // warps 0-7: tile arithmetic; warps 8, 9: copies, fences and flags
constexpr int kMath = 256;
constexpr int kPair = kMath + 32;  // the arithmetic warps and one copy warp (producer/consumer barriers)
constexpr int kTile = kB * kB;
constexpr int kPad = kB + 1;  // row stride of staged tiles (conflict-free column reads)
constexpr int kPadTile = kB * kPad;
constexpr int kMaxBlk = 24;                // block rows handled by the cluster solve (n <= 384)
constexpr unsigned long long kWaitNs = 1000000000ull;        // a wait on a worker's flag gives up after 1 s
constexpr unsigned long long kGuardWaitNs = 4000000000ull;   // the waits that guard shared memory, 4 s
constexpr unsigned kPollCap = 1u << 27;                      // polls per wait, should the timer stall

// named barriers (0 is __syncthreads)
constexpr int kBarPivot = 1;    // pivot chain and pivot application (160 threads)
constexpr int kBarMath = 2;     // warps 0-7
constexpr int kBarPanel = 3;    // chain CTA: panel result ready for warp 8
constexpr int kBarOutFull = 4;  // workers: result buffer b ready for warp 8, ids 4, 5
constexpr int kBarOutFree = 6;  // workers: result buffer b stored, ids 6, 7
constexpr int kBarInFull = 8;   // workers: inputs of the next task staged by warp 9, ids 8, 9
constexpr int kBarInFree = 10;  // workers: stage b read by warps 0-7, ids 10, 11
constexpr int kHelpers = 6;     // chain CTA, backward solve: warps 1-3 and 5-7 apply the terms of t

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

// Flag access at cluster scope (generic addresses into the chain CTA's
// shared memory, from any CTA of the cluster).
__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.cluster.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.cluster.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// This CTA's shared-memory address of `local`'s offset in cluster CTA `rank`.
__device__ __forceinline__ unsigned cluster_addr(const void* local, unsigned rank) {
  unsigned r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_u32(local)), "r"(rank));
  return r;
}

// Asynchronous 8-byte store into another CTA's shared memory; its arrival is
// counted in bytes on an mbarrier of that CTA.
__device__ __forceinline__ void st_async(unsigned raddr, double v, unsigned rbar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.f64 [%0], %1, [%2];" ::"r"(raddr), "d"(v),
               "r"(rbar)
               : "memory");
}

// Phase test with cluster-scope acquire (for data other CTAs stored).
__device__ __forceinline__ bool mbar_try_wait_cluster(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, "
      "p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait for *p >= v (one thread).  Returns false when the wait ran
// out (it then sets the abort word) or, unless guard, when another wait
// already ran out.  guard: the flag's producer runs whatever the abort word
// says, and the wait keeps waiting for it (up to kGuardWaitNs).  The abort
// word and the timer are read after the first failed poll and then once per
// 64 polls; the read after the first failed poll also spaces the polls (with
// back-to-back polls the factorisation measured 3% slower).
__device__ bool wait_ge(const int* p, int v, int* abort_word, bool guard = false) {
  unsigned long long t0 = 0;
  for (unsigned it = 0; it < kPollCap; ++it) {
    if (ld_acquire(p) >= v) return true;
    if ((it & 63u) == 0) {
      if (!guard && ld_acquire(abort_word) != 0) return false;
      const unsigned long long t = now_ns();
      if (it == 0)
        t0 = t;
      else if (t - t0 > (guard ? kGuardWaitNs : kWaitNs))
        break;
    }
    if (it > 32) __nanosleep(64);
  }
  st_release(abort_word, 1);
  return false;
}

// Counters in this CTA's shared memory that its warps hand over through
// (release / acquire at CTA scope).
__device__ __forceinline__ void st_local(int* p, int v) {
  asm volatile("st.release.cta.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(p)), "r"(v) : "memory");
}

__device__ __forceinline__ int ld_local(const int* p) {
  int v;
  asm volatile("ld.acquire.cta.shared::cta.b32 %0, [%1];" : "=r"(v) : "r"(smem_u32(p)) : "memory");
  return v;
}

// Bounded wait (every lane of a warp may call it) for *p >= v, a counter
// that another warp of this CTA advances whatever the abort word says; a
// wait that runs out sets the abort word.
__device__ void wait_local(const int* p, int v, int* abort_word) {
  unsigned long long t0 = 0;
  for (unsigned it = 0; it < kPollCap; ++it) {
    if (ld_local(p) >= v) return;
    if ((it & 63u) == 0) {
      const unsigned long long t = now_ns();
      if (it == 0)
        t0 = t;
      else if (t - t0 > kGuardWaitNs)
        break;
    }
  }
  st_release(abort_word, 1);
}

// The same for the phase the lookahead worker's pushes complete; that worker
// runs every push whatever the abort word says.
__device__ void mbar_wait_cluster(uint64_t* bar, unsigned parity, int* abort_word) {
  unsigned long long t0 = 0;
  for (unsigned it = 0; it < kPollCap; ++it) {
    if (mbar_try_wait_cluster(bar, parity)) return;
    if ((it & 63u) == 0) {
      const unsigned long long t = now_ns();
      if (it == 0)
        t0 = t;
      else if (t - t0 > kGuardWaitNs)
        break;
    }
  }
  st_release(abort_word, 1);
}

struct Geo {
  int C, nblk, ld, n;
  int hold;  // a flag the workers leave unreleased (-1 in every solve; the test of the bounded waits
             // sets it so that a wait runs out)
  // workspace (doubles): nblk x nblk tiles of 256, then the right-hand-side
  // rows W, 1/d and y (16 nblk each), then the inverses M_J (256 each,
  // transposed), then the products P_J = M_J L_{J+1,J}^T (256 each,
  // transposed), each part 256-byte aligned
  __host__ __device__ size_t tile_off(int i, int j) const { return ((size_t)i * nblk + j) * kTile; }
  __host__ __device__ size_t rhs_w() const { return (size_t)nblk * nblk * kTile; }
  __host__ __device__ size_t rhs_rd() const { return rhs_w() + (size_t)kB * nblk; }
  __host__ __device__ size_t rhs_y() const { return rhs_rd() + (size_t)kB * nblk; }
  __host__ __device__ size_t m_offset() const { return ((rhs_y() + (size_t)kB * nblk + 31) / 32) * 32; }
  __host__ __device__ size_t p_offset() const { return m_offset() + (size_t)nblk * kTile; }
  __host__ __device__ size_t ws_doubles() const { return p_offset() + (size_t)nblk * kTile; }
  // version flags (ints, in the chain CTA's shared memory): one per tile
  // ((nblk + 1) x nblk, right-hand-side row last), one per inverse M_J, and
  // the abort word
  __host__ __device__ int inv_index(int J) const { return (nblk + 1) * nblk + J; }
  __host__ __device__ int abort_index() const { return (nblk + 2) * nblk; }
  __host__ __device__ int flag_count() const { return (nblk + 2) * nblk + 1; }
  // chain CTA shared memory (doubles): two diagonal tiles with 1/d and the
  // squares of the sub-diagonal (step k factors tile D[k & 1] and receives
  // the next one in D[(k+1) & 1]), two incoming panel tiles (P[k & 1]), W
  // and L of the panel, the padded copy of L_kk with 1/d, and the two
  // mbarriers on which the next step's tiles arrive from a worker
  __host__ __device__ size_t c_diag(int b) const { return (size_t)b * (kTile + 2 * kB); }
  __host__ __device__ size_t c_p(int b) const { return 2 * (size_t)(kTile + 2 * kB) + (size_t)b * kTile; }
  __host__ __device__ size_t c_wp() const { return c_p(2); }
  __host__ __device__ size_t c_lp() const { return c_wp() + kPadTile; }
  __host__ __device__ size_t c_lk() const { return c_lp() + kPadTile; }
  __host__ __device__ size_t c_rx(int b) const { return c_lk() + kPadTile + kB + b; }
  __host__ __device__ size_t c_end() const { return c_rx(2); }
  // backward solve, after that: t, x, the counters its warps hand over
  // through (ints) and M of the last diagonal tile
  __host__ __device__ size_t b_t() const { return c_end(); }
  __host__ __device__ size_t b_x() const { return b_t() + (size_t)kB * nblk; }
  __host__ __device__ size_t b_fl() const { return b_x() + (size_t)kB * nblk; }
  __host__ __device__ size_t b_mlast() const { return b_fl() + (size_t)((((2 + nblk) + 1) / 2 + 1) & ~1); }
  __host__ __device__ size_t b_end() const { return b_mlast() + kTile; }
  // worker: two input stages (A, then W or L_kk, then L or 1/d) and two
  // result buffers of 512
  __host__ __device__ size_t w_stage(int b) const { return (size_t)b * (kTile + 2 * kPadTile); }
  __host__ __device__ size_t w_out(int b) const { return w_stage(2) + (size_t)b * 2 * kTile; }
  __host__ __device__ size_t w_end() const { return w_out(2); }
  // the flags, after everything the chain CTA uses (doubles)
  __host__ __device__ size_t f_base() const { return c_end() > b_end() ? c_end() : b_end(); }
  __host__ __device__ size_t total() const {
    const size_t t = f_base() + ((size_t)flag_count() + 1) / 2;
    return t > w_end() ? t : w_end();
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
__device__ __forceinline__ int* flag_at(int* fl, int nblk, int i, int j) { return fl + i * nblk + j; }

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

// ------------------------------------------------------------ chain CTA --

__device__ void chain_cta(const Geo& g, const double* S, double* ws, double* x, int* solve_ok, int* fl,
                          double* sm) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int rr = (tid >> 4) & 15, cc = tid & 15;
  const int nblk = g.nblk, ld = g.ld;
  int* abort_word = fl + g.abort_index();
  double* const Tb0 = sm + g.c_diag(0);
  double* const Tb1 = sm + g.c_diag(1);
  double* const P0 = sm + g.c_p(0);
  double* const P1 = sm + g.c_p(1);
  double* Wp = sm + g.c_wp();
  double* Lp = sm + g.c_lp();
  double* Lk = sm + g.c_lk();
  double* t = sm + g.b_t();
  double* xs = sm + g.b_x();
  double* const Mlast = sm + g.b_mlast();
  int cur = 0;
  if (tid < kMath) Tb0[tid] = __ldcg(S + (size_t)rr * ld + cc);
  __syncthreads();

  for (int k = 0; k + 1 < nblk; ++k) {
    double* T = cur ? Tb1 : Tb0;
    double* Q = cur ? Tb0 : Tb1;
    double* P = (k & 1) ? P1 : P0;
    // ---- (a) factor diagonal tile k; meanwhile tiles (k+1, k) and
    //      (k+1, k+1) at version k arrive in P and Q: pushed by the worker
    //      that ran their last updates, or, for k = 0, read from S by warp 8
    if (warp < 8) {
      if (warp < 4 || warp == 5) diag_ldlt(T, T + kTile, T + kTile + kB, solve_ok);
    } else if (warp == 8) {
      if (k > 0) {
        mbar_wait_cluster(reinterpret_cast<uint64_t*>(sm + g.c_rx(k & 1)), (unsigned)(((k - 1) >> 1) & 1),
                          abort_word);  // rx[1] serves steps 1, 3, .., rx[0] steps 2, 4, ..
      } else {
        double v[16];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int e = lane + 32 * u;
          v[u] = __ldcg(S + s_at(ld, nblk, 1, 0, e >> 4, e & 15));
          v[8 + u] = __ldcg(S + s_at(ld, nblk, 1, 1, e >> 4, e & 15));
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          P[lane + 32 * u] = v[u];
          Q[lane + 32 * u] = v[8 + u];
        }
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
      bar_arrive(kBarPanel, kPair);
      bar_sync(kBarMath, kMath);  // (c) reads rows of W and L written by other warps
    } else if (warp == 8) {
      // the bytes step k+1 receives are expected before the flag below lets
      // the worker push them: two tiles, or the right-hand-side row
      if (lane == 0)
        mbar_expect_tx(reinterpret_cast<uint64_t*>(sm + g.c_rx((k + 1) & 1)),
                       (k + 2 < nblk ? 2 * kTile : kB) * (unsigned)sizeof(double));
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int e = lane + 32 * u;
        if ((e >> 4) >= (e & 15)) __stcg(ws + g.tile_off(k, k) + e, T[e]);
      }
      if (lane < kB) __stcg(ws + g.rhs_rd() + kB * k + lane, T[kTile + lane]);
      __threadfence();
      __syncwarp();
      if (lane == 0) st_release(flag_at(fl, nblk, k, k), k + 1);
      bar_sync(kBarPanel, kPair);
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
  //      to shared memory for the backward solve and the last y into t.
  {
    const int k = nblk - 1;
    double* T = cur ? Tb1 : Tb0;
    double* P = (k & 1) ? P1 : P0;
    if (warp < 8) {
      if (warp < 4 || warp == 5) diag_ldlt(T, T + kTile, T + kTile + kB, solve_ok);
    } else if (warp == 8) {
      if (k > 0) {
        mbar_wait_cluster(reinterpret_cast<uint64_t*>(sm + g.c_rx(k & 1)), (unsigned)(((k - 1) >> 1) & 1),
                          abort_word);
      } else if (lane < kB) {
        P[lane] = __ldcg(S + s_at(ld, nblk, nblk, 0, 0, lane));
      }
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
      Mlast[c * kB + row] = m;  // M_k stored transposed
    } else if (warp == 8) {
      const double a = fwd_rows(lane < kB ? P[lane] : 0.0, Lk, lane);
      if (lane < kB) t[kB * k + lane] = a * Lk[kPadTile + lane];
    }
  }

  // ---- backward solve L^T x = y, block row by block row, as a dataflow
  //      inside the chain CTA.  x_J = M_J t_J - P_J x_{J+1}, where t_J must
  //      hold y_J minus the terms L_KJ^T x_K of every K >= J+2:
  //        warps 1-3, 5-7 (helpers): helper h owns the rows I = h mod 6 of
  //                 t and applies x_K's terms to them as x_K appears (K
  //                 descending; row K-2, needed next, first), then marks
  //                 row K-2 ready
  //        warp 4:  v_J = M_J t_J into t's row J once row J is ready
  //        warp 0:  P_J x_{J+1}, then x_J = v_J - P_J x_{J+1}
  //      (warps 0 and 4 share sub-partition 0, the helpers two to each of
  //      the others: so each sub-partition's FP64 pipe carries about the
  //      same number of products)
  //      The warps hand over through counters in shared memory (release /
  //      acquire at CTA scope): rows of x published, rows of v formed and a
  //      ready mark per row.  Each warp loads the tiles it multiplies by
  //      (P_J, M_J, L_KI) from L2 straight into registers, two rows or two
  //      terms ahead of their use, so no copy into shared memory paces the
  //      rows (bulk copies of the rows into shared memory took ~1.1 us a row
  //      to issue and land).  Warps 8 and 9 take no part after warp 8's
  //      waits below.  Every producer of the counters runs inside the CTA
  //      whatever the abort word says, so their waits do not end on it.
  //      Right-hand-side panel J is done only after every L_JI was (its
  //      updates read them), and the last right-hand-side tile waited above
  //      covers row nblk-1; so warp 8 waits for the right-hand-side panels
  //      and the inverses, one lane per row, before anything is read.
  int* const xcnt = reinterpret_cast<int*>(sm + g.b_fl());
  int* const vcnt = xcnt + 1;
  int* const ready = xcnt + 2;
  if (warp == 8) {
    if (lane < nblk - 1) {
      wait_ge(flag_at(fl, nblk, nblk, lane), lane + 1, abort_word);
      wait_ge(fl + g.inv_index(lane), 1, abort_word);
    }
  } else if (tid < 2 + nblk) {
    xcnt[tid] = 0;
  }
  __syncthreads();
  const int h = lane >> 4, c = lane & 15;
  // lane (h, c)'s eight elements of a transposed tile in the workspace
  // (global memory): [(8h + q) * 16 + c]
  auto load8 = [&](double* r, const double* tile) {
#pragma unroll
    for (int q = 0; q < 8; ++q) r[q] = __ldcg(tile + (8 * h + q) * kB + c);
  };
  const double* const Mg = ws + g.m_offset();
  const double* const Pg = ws + g.p_offset();
  // three register tiles per warp, in rotation: each load is made two rows
  // (or two terms) ahead of its use and used where it landed
  double b0[8] = {}, b1[8] = {}, b2[8] = {};
  // warp 0: P_{nblk-2} and P_{nblk-3}; warp 4: M_{nblk-2} and M_{nblk-3}
  // (M_{nblk-1} the chain CTA formed in shared memory)
  if (warp == 0 || warp == 4) {
    const double* base = warp == 0 ? Pg : Mg;
    if (nblk >= 2) load8(b0, base + (size_t)(nblk - 2) * kTile);
    if (nblk >= 3) load8(b1, base + (size_t)(nblk - 3) * kTile);
  }
  for (int e = tid; e < kB * (nblk - 1); e += kThreads) t[e] = __ldcg(ws + g.rhs_y() + e);
  __syncthreads();
  const bool write_x = *(volatile int*)solve_ok != 0;  // every pivot is known by now
  if (warp == 0) {
    // x_J = v_J - P_J x_{J+1} (no P for the last row)
    auto row = [&](const double(&Pr)[8], int J) {
      double y = 0.0;
      if (J + 1 < nblk) {
        const double* xj = xs + kB * (J + 1);
        double p0 = 0.0, p1 = 0.0;
#pragma unroll
        for (int q = 0; q < 8; q += 2) {
          p0 = fma(Pr[q], xj[8 * h + q], p0);
          p1 = fma(Pr[q + 1], xj[8 * h + q + 1], p1);
        }
        y = p0 + p1;
        y += __shfl_xor_sync(0xffffffffu, y, 16);
      }
      wait_local(vcnt, nblk - J, abort_word);  // v_J is in t's row J
      if (lane < kB) {
        const double xv = t[kB * J + c] - y;
        xs[kB * J + c] = xv;
        if (kB * J + c < g.n && write_x) x[kB * J + c] = xv;
      }
      __syncwarp();
      if (lane == 0) st_local(xcnt, nblk - J);
    };
    // row J with P_J in cur; P_{J-2} into pre
    auto step = [&](const double(&cur)[8], double(&pre)[8], int J) {
      if (J < 0) return false;
      if (J >= 2) load8(pre, Pg + (size_t)(J - 2) * kTile);
      row(cur, J);
      return true;
    };
    row(b2, nblk - 1);
    for (int J = nblk - 2; step(b0, b2, J) && step(b1, b0, J - 1) && step(b2, b1, J - 2); J -= 3) {
    }
  } else if (warp == 4) {
    // v_J = M_J t_J into t's row J once row J is ready
    auto row = [&](const double(&Mr)[8], int J) {
      if (J + 2 < nblk) wait_local(ready + J, 1, abort_word);
      const double u = t[kB * J + c];
      double p0 = 0.0, p1 = 0.0;
#pragma unroll
      for (int q = 0; q < 8; q += 2) {
        const double u0 = __shfl_sync(0xffffffffu, u, 8 * h + q);
        const double u1 = __shfl_sync(0xffffffffu, u, 8 * h + q + 1);
        p0 = fma(Mr[q], u0, p0);
        p1 = fma(Mr[q + 1], u1, p1);
      }
      double v = p0 + p1;
      v += __shfl_xor_sync(0xffffffffu, v, 16);
      if (lane < kB) t[kB * J + c] = v;
      __syncwarp();
      if (lane == 0) st_local(vcnt, nblk - J);
    };
    auto step = [&](const double(&cur)[8], double(&pre)[8], int J) {
      if (J < 0) return false;
      if (J >= 2) load8(pre, Mg + (size_t)(J - 2) * kTile);
      row(cur, J);
      return true;
    };
    {  // M_{nblk-1} from shared memory
      const double* Ms = Mlast;
#pragma unroll
      for (int q = 0; q < 8; ++q) b2[q] = Ms[(8 * h + q) * kB + c];
      row(b2, nblk - 1);
    }
    for (int J = nblk - 2; step(b0, b2, J) && step(b1, b0, J - 1) && step(b2, b1, J - 2); J -= 3) {
    }
  } else if (warp < 8) {
    const int hw = warp < 4 ? warp - 1 : warp - 2;  // helper 0..5: sub-partitions 1, 2, 3, 1, 2, 3
    // this helper's terms (K, I): K = nblk-1 .. 2, its rows I <= K-2
    // descending; advance to the term after (K, I) (I = -1: none left)
    auto next = [&](int& K, int& I) {
      if (I >= kHelpers) {
        I -= kHelpers;
        return;
      }
      for (--K; K >= 2; --K)
        if (K - 2 >= hw) {
          I = K - 2 - (K - 2 - hw) % kHelpers;
          return;
        }
      I = -1;
    };
    // the current term, the next two
    int Kc = nblk, Ic = -1;
    next(Kc, Ic);
    int K1 = Kc, I1 = Ic;
    if (I1 >= 0) next(K1, I1);
    if (Ic >= 0) load8(b0, ws + g.tile_off(Ic, Kc));  // L_KI^T[c][q] at [q * 16 + c]
    if (I1 >= 0) load8(b1, ws + g.tile_off(I1, K1));
    int Kx = nblk;
    double xk[8];
    auto step = [&](const double(&cur)[8], double(&pre)[8]) {
      if (Ic < 0) return false;
      int K2 = K1, I2 = I1;
      if (I2 >= 0) next(K2, I2);
      if (I2 >= 0) load8(pre, ws + g.tile_off(I2, K2));
      if (Kc != Kx) {  // the first term of x_K: wait for it
        Kx = Kc;
        wait_local(xcnt, nblk - Kc, abort_word);
#pragma unroll
        for (int q = 0; q < 8; ++q) xk[q] = xs[kB * Kc + 8 * h + q];
      }
      double p0 = 0.0, p1 = 0.0;
#pragma unroll
      for (int q = 0; q < 8; q += 2) {
        p0 = fma(cur[q], xk[q], p0);
        p1 = fma(cur[q + 1], xk[q + 1], p1);
      }
      double sum = p0 + p1;
      sum += __shfl_xor_sync(0xffffffffu, sum, 16);
      if (lane < kB) t[kB * Ic + c] -= sum;
      if (Ic == Kc - 2) {  // row K-2 has all its terms
        __syncwarp();
        if (lane == 0) st_local(ready + Ic, 1);
      }
      Kc = K1;
      Ic = I1;
      K1 = K2;
      I1 = I2;
      return true;
    };
    while (step(b0, b2) && step(b1, b0) && step(b2, b1)) {
    }
  }
  __syncthreads();
  if (tid == 0 && ld_acquire(abort_word) != 0) *solve_ok = 0;
}

// --------------------------------------------------------------- workers --
//
// A worker runs its tasks as a three-stage pipeline: warp 9 waits for a
// task's inputs and stages them in shared memory (stage b = task parity),
// warps 0-7 compute the result into result buffer b, and warp 8 stores the
// result, fences it and releases its flag.  So flag waits, L2 loads and
// fences overlap the arithmetic of the neighbouring tasks.  Task kinds:
//   panel (i, k): inputs tile (i, k) at version k, L_kk and 1/d_k; W to tile
//                 (i, k), L to tile (k, i) (the right-hand side: the W and y
//                 rows), flag (i, k) = k+1
//   update (i, j, s): inputs tile (i, j) at version s, W_is, L_js; result to
//                 tile (i, j) (lower part of a diagonal tile, row 0 of the
//                 right-hand side), flag (i, j) = s+1
//   inverse J:    inputs L_JJ and L_{J+1,J}; M_J = L_JJ^-T and
//                 P_J = M_J L_{J+1,J}^T to theirs, inverse flag J = 1
//   lookahead (r, s+1, s), right after panel (r, s), r = s+2: step s on
//                 tiles (r, s+1) and (r, r) with W and L of that panel; the
//                 two tiles are the chain CTA's inputs for step s+1 and go
//                 straight into its shared memory (st.async, counted on its
//                 mbarrier), not to the workspace
enum : int { kTaskPanel = 0, kTaskUpdate = 1, kTaskInv = 2, kTaskLook = 3 };

// Stage layout (doubles): A (16 x 16), then W (or L_kk) and L, padded.
constexpr int kStA = 0;
constexpr int kStW = kTile;
constexpr int kStL = kTile + kPadTile;
constexpr int kStRd = kTile + kPadTile;  // 1/d of a panel's L_kk (the L slot is free)

// Warp 9: a 16x16 tile (or only its row 0) at version v into shared memory,
// two elements per load.
__device__ __forceinline__ void stage_tile(const Geo& g, const double* S, const double* ws, int i, int j,
                                           int v, double* dst, int stride, bool row0) {
  const int lane = threadIdx.x & 31;
  double2 a[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int e = 2 * (lane + 32 * u), rr = e >> 4, cc = e & 15;
    a[u] = make_double2(0.0, 0.0);
    if (!row0 || rr == 0) {
      if (v == 0)
        a[u] = __ldcg(reinterpret_cast<const double2*>(S + s_at(g.ld, g.nblk, i, j, rr, cc)));
      else
        a[u] = __ldcg(reinterpret_cast<const double2*>(ws + w_at(g, i, j, rr, cc)));
    }
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int e = 2 * (lane + 32 * u), rr = e >> 4, cc = e & 15;
    if (!row0 || rr == 0) {
      dst[rr * stride + cc] = a[u].x;
      dst[rr * stride + cc + 1] = a[u].y;
    }
  }
}

// Warp 9: wait for task (kind, i, j, s)'s producers, then stage its inputs.
__device__ void load_task(const Geo& g, const double* S, const double* ws, int* fl, double* st, int kind,
                          int i, int j, int s) {
  const int lane = threadIdx.x & 31;
  const int nblk = g.nblk;
  int* abort_word = fl + g.abort_index();
  int* f = nullptr;
  int v = 0;
  bool guard = false;
  if (kind == kTaskPanel) {  // (i, k = j) at version k, diagonal tile k factored
    if (lane == 0 && j > 0) f = flag_at(fl, nblk, i, j), v = j;
    if (lane == 1) f = flag_at(fl, nblk, j, j), v = j + 1;
  } else if (kind == kTaskUpdate) {  // tile at version s, panels (i, s) and (j, s)
    if (lane == 0 && s > 0) f = flag_at(fl, nblk, i, j), v = s;
    if (lane == 1) f = flag_at(fl, nblk, i, s), v = s + 1;
    if (lane == 2) f = flag_at(fl, nblk, j, s), v = s + 1;
  } else if (kind == kTaskLook) {  // tiles (i, j = s+1) and (i, i) at version s, the chain's panel (s+1, s)
    if (lane == 0 && s > 0) f = flag_at(fl, nblk, i, j), v = s;
    if (lane == 1 && s > 0 && i < nblk) f = flag_at(fl, nblk, i, i), v = s;
    // the chain CTA releases its panel after arming the mbarrier the pushes
    // count on and after its last read of the buffers they overwrite
    if (lane == 2) f = flag_at(fl, nblk, j, s), v = s + 1, guard = true;
  } else {  // diagonal tile i factored, the chain's panel (i+1, i)
    if (lane == 0) f = flag_at(fl, nblk, i, i), v = i + 1;
    if (lane == 1 && i + 1 < nblk) f = flag_at(fl, nblk, i + 1, i), v = i + 1;
  }
  if (f) wait_ge(f, v, abort_word, guard);
  __syncwarp();
  if (kind == kTaskPanel) {
    stage_tile(g, S, ws, i, j, j, st + kStA, kB, i == nblk);
    stage_tile(g, S, ws, j, j, 1, st + kStW, kPad, false);
    if (lane < kB) st[kStRd + lane] = __ldcg(ws + g.rhs_rd() + kB * j + lane);
  } else if (kind == kTaskUpdate) {
    stage_tile(g, S, ws, i, j, s, st + kStA, kB, i == nblk);
    stage_tile(g, S, ws, i, s, 1, st + kStW, kPad, i == nblk);
    stage_tile(g, S, ws, s, j, 1, st + kStL, kPad, false);  // L_js sits in the upper tile (s, j)
  } else if (kind == kTaskLook) {
    stage_tile(g, S, ws, i, j, s, st + kStA, kB, i == nblk);
    if (i < nblk) stage_tile(g, S, ws, i, i, s, st + kStW, kB, false);
    stage_tile(g, S, ws, s, j, 1, st + kStL, kPad, false);
  } else {
    stage_tile(g, S, ws, i, i, 1, st + kStW, kPad, false);
    if (i + 1 < nblk) stage_tile(g, S, ws, i, i + 1, 1, st + kStL, kPad, false);  // L_{i+1,i}
  }
}

// Warps 0-7: the result of a staged task into out (512 doubles); prev is
// the previous task's result (the panel a lookahead task continues).
__device__ void math_task(const Geo& g, const double* st, double* out, const double* prev, double* sm, int kind,
                          int i, int j) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool rhs = (i == g.nblk);
  const double* Lk = st + kStW;
  if (kind == kTaskLook) {
    // tile (i, j) -= W L_{j,j-1}^T and tile (i, i) -= W L^T (lower part),
    // W and L of panel (i, j-1) in prev; L goes to out, padded, first
    const int rr = tid >> 4, cc = tid & 15;
    out[rr * kPad + cc] = prev[kTile + tid];
    bar_sync(kBarMath, kMath);
    const double* wr = prev + rr * kB;
    const double* l1 = st + kStL + cc * kPad;
    const double* l2 = out + cc * kPad;
    double a0 = 0.0, a1 = 0.0, b0 = 0.0, b1 = 0.0;
#pragma unroll
    for (int q = 0; q < kB; q += 2) {
      a0 = fma(wr[q], l1[q], a0);
      a1 = fma(wr[q + 1], l1[q + 1], a1);
      b0 = fma(wr[q], l2[q], b0);
      b1 = fma(wr[q + 1], l2[q + 1], b1);
    }
    // into the chain CTA: P[j & 1] and D[(j+1) & 1], counted on its mbarrier
    // rx[j & 1]
    const unsigned rbar = cluster_addr(sm + g.c_rx(j & 1), 0);
    if (!rhs || rr == 0) st_async(cluster_addr(sm + g.c_p(j & 1) + tid, 0), st[kStA + tid] - (a0 + a1), rbar);
    if (!rhs)
      st_async(cluster_addr(sm + g.c_diag((j + 1) & 1) + tid, 0), rr >= cc ? st[kStW + tid] - (b0 + b1) : 0.0, rbar);
    return;
  }
  if (kind == kTaskPanel) {
    // W = A L_kk^-T (two rows per warp), L = W D_k^-1
    const int row = 2 * warp + (lane >> 4), c = lane & 15;
    if (!rhs || warp == 0) {
      const double a = fwd_rows((!rhs || row == 0) ? st[kStA + row * kB + c] : 0.0, Lk, lane);
      out[row * kB + c] = a;
      out[kTile + row * kB + c] = a * st[kStRd + c];
    }
  } else if (kind == kTaskUpdate) {
    // A_ij -= W_is L_js^T (lower part of a diagonal tile, row 0 of the
    // right-hand side)
    const int rr = tid >> 4, cc = tid & 15;
    if (rhs ? rr == 0 : (i != j || rr >= cc)) {
      const double* wr = st + kStW + rr * kPad;
      const double* lc = st + kStL + cc * kPad;
      double s0 = 0.0, s1 = 0.0;
#pragma unroll
      for (int q = 0; q < kB; q += 2) {
        s0 = fma(wr[q], lc[q], s0);
        s1 = fma(wr[q + 1], lc[q + 1], s1);
      }
      out[tid] = st[kStA + tid] - (s0 + s1);
    }
  } else {
    // M_J = L_JJ^-T, the panel solve of the identity, stored transposed
    // (M_J[c][q] at [q * 16 + c]); then P_J = M_J L_{J+1,J}^T, stored the
    // same way, into the second half
    const int row = 2 * warp + (lane >> 4), c = lane & 15;
    out[c * kB + row] = fwd_rows(row == c ? 1.0 : 0.0, Lk, lane);
    if (i + 1 < g.nblk) {
      bar_sync(kBarMath, kMath);
      const int q = tid >> 4, cc = tid & 15;
      const double* lq = st + kStL + q * kPad;  // row q of L_{J+1,J}
      double p0 = 0.0, p1 = 0.0;
#pragma unroll
      for (int r = 0; r < kB; r += 2) {
        p0 = fma(out[r * kB + cc], lq[r], p0);
        p1 = fma(out[(r + 1) * kB + cc], lq[r + 1], p1);
      }
      out[kTile + tid] = p0 + p1;
    }
  }
}

// Warp 8: store a result, fence it and release its flag.
__device__ void store_task(const Geo& g, double* ws, int* fl, const double* out, int kind, int i, int j, int s) {
  const int lane = threadIdx.x & 31;
  const int nblk = g.nblk;
  if (kind == kTaskLook) return;  // went to the chain CTA directly
  int* f = nullptr;
  int v = 0;
  if (kind == kTaskPanel) {
    if (i < nblk) {
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int e = 2 * (lane + 32 * u);
        __stcg(reinterpret_cast<double2*>(ws + g.tile_off(i, j) + e), *reinterpret_cast<const double2*>(out + e));
        __stcg(reinterpret_cast<double2*>(ws + g.tile_off(j, i) + e),
               *reinterpret_cast<const double2*>(out + kTile + e));
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
    for (int u = 0; u < 4; ++u) {
      const int e = 2 * (lane + 32 * u);
      __stcg(reinterpret_cast<double2*>(ws + g.m_offset() + (size_t)i * kTile + e),
             *reinterpret_cast<const double2*>(out + e));
      if (i + 1 < nblk)
        __stcg(reinterpret_cast<double2*>(ws + g.p_offset() + (size_t)i * kTile + e),
               *reinterpret_cast<const double2*>(out + kTile + e));
    }
    f = fl + g.inv_index(i);
    v = 1;
  }
  __threadfence();
  __syncwarp();
  if (lane == 0 && (int)(f - fl) != g.hold) st_release(f, v);
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

// Calls f(kind, i, j, s) for this worker's tasks in order.  Worker 1 runs
// only the lookahead rows, so it is idle when the chain CTA publishes the
// diagonal tile they wait for; the other tasks are dealt over workers
// 2..C-1.
template <typename F>
__device__ void worker_tasks(const Geo& g, int rank, F&& f) {
  const int nblk = g.nblk;
  if (rank == 1) {
    // (0) block row k+2, the chain CTA's next input: its panel, then step k
    //     on its tiles (k+2, k+1) and (k+2, k+2); then, while the chain CTA
    //     factors tile k+1, the backward-solve inverse of diagonal tile k
    for (int k = 0; k + 2 <= nblk; ++k) {
      f(kTaskPanel, k + 2, k, k);
      f(kTaskLook, k + 2, k + 1, k);
      f(kTaskInv, k, k, 0);
    }
    return;
  }
  Deal d{g.C - 2, rank - 2, 0};
  for (int k = 0; k < nblk; ++k) {
    // (1) the other panels (i, k), i >= k+3, right-hand side last (the last
    //     column's right-hand-side panel is the chain CTA's)
    if (k + 1 < nblk) d.segment(nblk - k - 2, [&](int idx) { f(kTaskPanel, k + 3 + idx, k, k); });
    // (2) step k on block column k+1 below (the chain CTA updates the
    //     diagonal tile itself)
    if (k + 1 < nblk) d.segment(nblk - k - 2, [&](int idx) { f(kTaskUpdate, k + 3 + idx, k + 1, k); });
    // (3) step k on block column k+2 below
    if (k + 2 < nblk) d.segment(nblk - k - 2, [&](int idx) { f(kTaskUpdate, k + 3 + idx, k + 2, k); });
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
  }
}

__device__ void worker_cta(const Geo& g, const double* S, double* ws, int* fl, double* sm, int rank) {
  const int warp = threadIdx.x >> 5;
  int n = 0;  // tasks so far; stage and result buffer n & 1
  if (warp < 8) {
    worker_tasks(g, rank, [&](int kind, int i, int j, int s) {
      const int b = n & 1;
      bar_sync(kBarInFull + b, kPair);                   // warp 9 has staged task n
      if (n >= 2) bar_sync(kBarOutFree + b, kPair);      // warp 8 has stored task n-2
      math_task(g, sm + g.w_stage(b), sm + g.w_out(b), sm + g.w_out(b ^ 1), sm, kind, i, j);
      bar_arrive(kBarInFree + b, kPair);
      bar_arrive(kBarOutFull + b, kPair);
      ++n;
    });
    // balance warp 8's last two releases
    for (int q = max(n - 2, 0); q < n; ++q) bar_sync(kBarOutFree + (q & 1), kPair);
  } else if (warp == 8) {
    worker_tasks(g, rank, [&](int kind, int i, int j, int s) {
      const int b = n & 1;
      bar_sync(kBarOutFull + b, kPair);
      store_task(g, ws, fl, sm + g.w_out(b), kind, i, j, s);
      bar_arrive(kBarOutFree + b, kPair);
      ++n;
    });
  } else {
    worker_tasks(g, rank, [&](int kind, int i, int j, int s) {
      const int b = n & 1;
      if (n >= 2) bar_sync(kBarInFree + b, kPair);  // warps 0-7 are done with task n-2's stage
      load_task(g, S, ws, fl, sm + g.w_stage(b), kind, i, j, s);
      bar_arrive(kBarInFull + b, kPair);
      ++n;
    });
    for (int q = max(n - 2, 0); q < n; ++q) bar_sync(kBarInFree + (q & 1), kPair);
  }
}

inline Geo make_geo(int C, int ld, int n) {
  Geo g{};
  g.C = C;
  g.nblk = (n + kB - 1) / kB;
  g.ld = ld;
  g.n = n;
  g.hold = -1;
  return g;
}

// One solve by the calling cluster: every CTA of the cluster (kThreads
// threads each, sm its dynamic shared memory of at least g.total() doubles)
// calls this together.
__device__ __forceinline__ void ldlt_cluster_run(const double* S, double* ws, double* x, int* solve_ok, const Geo& g,
                                                 double* sm) {
  cg::cluster_group cl = cg::this_cluster();
  const int r = (int)cl.block_rank();
  // the flags in the chain CTA's shared memory, seen through the cluster's
  // shared-memory window
  int* const fl_local = reinterpret_cast<int*>(sm + g.f_base());
  int* fl = cl.map_shared_rank(fl_local, 0);
  // the chain CTA's receive mbarriers are ready before any worker can push
  if (r == 0 && threadIdx.x == kMath) {
    mbar_init(reinterpret_cast<uint64_t*>(sm + g.c_rx(0)), 1);
    mbar_init(reinterpret_cast<uint64_t*>(sm + g.c_rx(1)), 1);
    fence_mbar_init();
  }
  // the version flags and the abort word start at zero in every solve
  if (r == 0)
    for (int e = (int)threadIdx.x; e < g.flag_count(); e += kThreads) fl_local[e] = 0;
  cl.sync();
  if (r == 0)
    chain_cta(g, S, ws, x, solve_ok, fl, sm);
  else
    worker_cta(g, S, ws, fl, sm, r);
  // the chain CTA's shared memory holds the flags: it stays until every CTA
  // is past its last flag access (a wait that gave up may leave a worker
  // behind the chain CTA)
  cl.sync();
}

// After ldlt_cluster_run, for a caller that goes on to use the same shared
// memory otherwise (the next solve may have another geometry): the chain
// CTA's mbarriers are invalidated, and the thread's generic accesses are
// ordered before later asynchronous-proxy writes into its shared memory.
__device__ __forceinline__ void ldlt_cluster_retire(const Geo& g, double* sm, int rank) {
  if (rank == 0 && threadIdx.x == kMath) {
    mbar_inval(reinterpret_cast<uint64_t*>(sm + g.c_rx(0)));
    mbar_inval(reinterpret_cast<uint64_t*>(sm + g.c_rx(1)));
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

}  // namespace
}  // namespace chold
}  // namespace mcba
