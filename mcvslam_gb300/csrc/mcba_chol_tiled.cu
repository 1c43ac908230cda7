// mcba_chol_tiled.cu -- blocked FP64 Cholesky of larger reduced camera
// systems (LinearSolverEigen's LLT role, linear_solver_eigen.h:87-128), with
// the forward substitution carried along as an extra row and a blocked
// backward substitution.
//
// FP64 runs at about two FMA per clock per SM on this part (one warp
// instruction per ~58 cycles per SM sub-partition, and as much latency), so
// the work is spread over every SM and the critical path is kept short.
// Panels are 32 columns wide:
//   k_tchol_diag     one CTA: LDL^T pivot chain of diagonal tile k in shared
//                    memory (one barrier per pivot; the next pivot's
//                    reciprocal formed beside the live-entry updates), then
//                    L_kk = L_unit D^1/2 and 1 / L_jj, stored in ws
//   k_tchol_trsm     rows below tile k, the b row included: x L_kk^T = a, one
//                    warp per row, two rows interleaved
//   k_tchol_update   A_ij -= L_ik L_jk^T on strips of RH rows x 32 columns of
//                    the lower triangle (and of the b row), the panel staged
//                    in shared memory
//   k_tchol_tinv     after the factorisation: M_J = L_JJ^-1 of every diagonal
//                    tile, one CTA each, all at once
//   k_tchol_bsolve   one launch per block row I, from the last: x_I =
//                    M_I^T (y_I - t_I) (each CTA forms it), then every thread
//                    adds L_I,c^T x_I to the partial t_c of its column c < 32 I
// Lookahead: the update of the next panel's columns and that panel's
// diagonal tile and triangular solve run on the caller's stream while the
// update of the columns beyond runs on a side stream, at the lowest priority;
// the caller's stream waits for that update before it touches those columns.

#include <cuda_runtime.h>

#include "mcba_chol_tiled.h"
#include "mcba_device.cuh"

namespace mcba {
namespace {

constexpr int kTB = 32;  // panel width
constexpr int kTC = 32;  // column tile of the trailing update
constexpr int kDiagThreads = 256;
constexpr int kTri = kTB * (kTB + 1) / 2;

// Reciprocal of a pivot: rcp.approx.ftz.f64, then one cubic Newton-Raphson
// step y (1 + e + e^2), e = 1 - d y; values whose reciprocal leaves the normal
// range take the IEEE division.  That path is a separate, never-inlined call
// behind an unlikely branch: predicated in line, its instructions would run
// on every pivot of the chain.
__device__ __noinline__ double tchol_recip_ieee(double d) { return 1.0 / d; }
__device__ __noinline__ double tchol_rsqrt_ieee(double d) { return 1.0 / sqrt(d); }

__device__ __forceinline__ double tchol_recip(double d) {
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(d));
  const unsigned ex = ((unsigned)(__double_as_longlong(d) >> 52)) & 0x7ffu;
  if (__builtin_expect(ex < 0x040u || ex > 0x7bfu, 0)) return tchol_recip_ieee(d);
  const double e = fma(-d, y, 1.0);
  const double p = fma(e, e, e);
  return fma(y, p, y);
}

// 1 / sqrt(d): float estimate and two Newton-Raphson steps (as
// dev::rsqrt_newton), with the out-of-range path kept out of line.
__device__ __forceinline__ double tchol_rsqrt(double d) {
  if (__builtin_expect(!(d > 1e-36 && d < 1e36), 0)) return tchol_rsqrt_ieee(d);
  double y = (double)rsqrtf((float)d);
  const double hd = 0.5 * d;
  y = y * (1.5 - hd * y * y);
  y = y * (1.5 - hd * y * y);
  return y;
}

// ws layout (doubles): L_kk [nt][32][32] | M_k [nt][32][32] | t [ld]
// (backward-substitution partials) | 1 / L_jj [ld]; nt = ld / 32
__host__ __device__ inline size_t ws_L(int k) { return (size_t)k * kTB * kTB; }
__host__ __device__ inline size_t ws_M(int nt, int k) { return (size_t)(nt + k) * kTB * kTB; }
__host__ __device__ inline size_t ws_t(int nt) { return (size_t)2 * nt * kTB * kTB; }
__host__ __device__ inline size_t ws_r(int nt) { return ws_t(nt) + (size_t)nt * kTB; }

// Live entries of pivot kk: the trailing triangle (kk < j <= i < 32), listed
// row by row as (a, b) = (i - kk - 1, j - kk - 1) with b <= a; the list of a
// smaller triangle is a prefix of the list of a larger one.
__device__ __forceinline__ void tri_decode(int e, int& a, int& b) {
  a = (int)((sqrtf(8.f * (float)e + 1.f) - 1.f) * 0.5f);
  if ((a + 1) * (a + 2) / 2 <= e) ++a;  // float rounding guard
  if (a * (a + 1) / 2 > e) --a;
  b = e - a * (a + 1) / 2;
}

__global__ void __launch_bounds__(kDiagThreads) k_tchol_diag(const double* __restrict__ S, double* ws, int ld,
                                                              int k, int* solve_ok) {
  __shared__ double T[kTB][kTB + 1];
  __shared__ double dinv[kTB], rs[kTB], w2[kTB];
  __shared__ unsigned char ta[kTri], tb[kTri];
  const int tid = threadIdx.x, o = k * kTB, nt = ld / kTB;
  for (int idx = tid; idx < kTB * kTB; idx += kDiagThreads) {
    const int i = idx / kTB, j = idx % kTB;
    T[i][j] = (j <= i) ? S[(size_t)(o + i) * ld + o + j] : 0.0;
  }
  for (int e = tid; e < kTri; e += kDiagThreads) {
    int a, b;
    tri_decode(e, a, b);
    ta[e] = (unsigned char)a;
    tb[e] = (unsigned char)b;
  }
  __syncthreads();
  if (tid == 0) {
    const double d = T[0][0];
    if (!(d > 0.0)) *solve_ok = 0;
    dinv[0] = tchol_recip(d);
    w2[0] = T[1][0] * T[1][0];
  }
  __syncthreads();
  // LDL^T, one barrier per pivot.  At pivot kk the next pivot is
  // d_{kk+1} - w^2 / d_kk with w = T[kk+1][kk], whose square was formed at
  // the previous pivot (by the thread that wrote w), so the chain from one
  // reciprocal to the next is one FMA and the reciprocal itself.  Thread 0
  // runs that chain and nothing else, and no other FP64 work shares its
  // warp's sub-partition: the other live entries go to warps 1-3 and 5-7
  // (warp 4 is on warp 0's sub-partition and idles).  After pivot kk,
  // column kk below the diagonal holds L_unit[i][kk] d_kk.
  const int warp = tid >> 5;
  const int wk = (warp == 0 || warp == 4) ? -1 : (warp < 4 ? tid - 32 : tid - 64);  // 0..191
  constexpr int kWorkers = kDiagThreads - 64;
  for (int kk = 0; kk < kTB - 1; ++kk) {
    const int m = kTB - 1 - kk, live = m * (m + 1) / 2;
    const double inv = dinv[kk];
    if (tid == 0) {  // (kk+1, kk+1): the next pivot
      const double v = fma(-w2[kk], inv, T[kk + 1][kk + 1]);
      T[kk + 1][kk + 1] = v;
      if (!(v > 0.0)) *solve_ok = 0;  // SimplicialLLT's info() != Success (linear_solver_eigen.h:118-126)
      dinv[kk + 1] = tchol_recip(v);
    } else if (wk >= 0) {
      for (int e = 1 + wk; e < live; e += kWorkers) {
        const int i = kk + 1 + ta[e], j = kk + 1 + tb[e];
        const double v = fma(-(T[i][kk] * inv), T[j][kk], T[i][j]);
        T[i][j] = v;
        if (e == 1 && kk + 1 < kTB - 1) w2[kk + 1] = v * v;  // (kk+2, kk+1): w of the next pivot
      }
    }
    __syncthreads();
  }
  // L = L_unit D^1/2: L_ij = T_ij / sqrt(d_j), L_jj = sqrt(d_j)
  if (tid < kTB) rs[tid] = tchol_rsqrt(T[tid][tid]);
  __syncthreads();
  double* Lo = ws + ws_L(k);
  for (int idx = tid; idx < kTB * kTB; idx += kDiagThreads) {
    const int r = idx / kTB, c = idx % kTB;
    Lo[idx] = (c <= r) ? T[r][c] * rs[c] : 0.0;
  }
  if (tid < kTB) ws[ws_r(nt) + o + tid] = rs[tid];  // 1 / L_jj
}

// M_J = L_JJ^-1 of every diagonal tile, one CTA each, after the
// factorisation (only the backward substitution uses them): forward
// substitution of L M = I, row l final at step l.  Dynamic shared memory:
// L and M, 32 x 33 doubles each.
constexpr size_t kTinvSmem = 2 * sizeof(double) * kTB * (kTB + 1) + sizeof(double) * kTB;

__global__ void __launch_bounds__(kDiagThreads) k_tchol_tinv(double* ws, int ld) {
  extern __shared__ double dsm[];
  double(*T)[kTB + 1] = reinterpret_cast<double(*)[kTB + 1]>(dsm);
  double(*Mi)[kTB + 1] = reinterpret_cast<double(*)[kTB + 1]>(dsm + kTB * (kTB + 1));
  double* rs = dsm + 2 * kTB * (kTB + 1);
  const int tid = threadIdx.x, J = blockIdx.x, nt = ld / kTB;
  const double* Lk = ws + ws_L(J);
  for (int idx = tid; idx < kTB * kTB; idx += kDiagThreads) {
    const int i = idx / kTB, j = idx % kTB;
    T[i][j] = Lk[idx];
    Mi[i][j] = (i == j) ? 1.0 : 0.0;
  }
  if (tid < kTB) rs[tid] = ws[ws_r(nt) + J * kTB + tid];
  __syncthreads();
  for (int l = 0; l < kTB; ++l) {
    if (tid <= l) Mi[l][tid] *= rs[l];
    __syncthreads();
    const int cnt = (kTB - 1 - l) * (l + 1);
    for (int e = tid; e < cnt; e += kDiagThreads) {
      const int i = l + 1 + e / (l + 1), j = e % (l + 1);
      Mi[i][j] = fma(-T[i][l], Mi[l][j], Mi[i][j]);
    }
    __syncthreads();
  }
  double* Mo = ws + ws_M(nt, J);
  for (int idx = tid; idx < kTB * kTB; idx += kDiagThreads) {
    const int r = idx / kTB, c = idx % kTB;
    Mo[idx] = (c <= r) ? Mi[r][c] : 0.0;
  }
}

// Rows R in [o + kTB, nrows): row segment a (kTB values of panel k)
// becomes x with x L_kk^T = a.  One warp per row pair, lane l holding entry
// l (and l + 32 for 64-wide panels): a_m -= a_j (L_mj / L_jj) for m > j,
// then x_m = a_m / L_mm once at the end, so the dependent chain per column
// is one shuffle and one FMA.  Eight rows per CTA; the two rows of a warp
// run interleaved.  L_kk with its columns scaled by 1 / L_jj in dynamic
// shared memory.
constexpr size_t kTrsmSmem = sizeof(double) * kTB * (kTB + 1) + sizeof(double) * kTB;

__global__ void __launch_bounds__(128) k_tchol_trsm(double* S, const double* __restrict__ ws, int ld, int k,
                                                     int nrows) {
  extern __shared__ double dsm[];
  double(*Ls)[kTB + 1] = reinterpret_cast<double(*)[kTB + 1]>(dsm);
  double* ri = dsm + kTB * (kTB + 1);
  const int tid = threadIdx.x, o = k * kTB, nt = ld / kTB;
  const double* Lk = ws + ws_L(k);
  if (tid < kTB) ri[tid] = ws[ws_r(nt) + o + tid];
  __syncthreads();
  for (int idx = tid; idx < kTB * kTB; idx += 128) Ls[idx / kTB][idx % kTB] = Lk[idx] * ri[idx % kTB];
  __syncthreads();
  const int lane = tid & 31, w = tid >> 5;
  const int R0 = o + kTB + blockIdx.x * 8 + w * 2, R1 = R0 + 1;
  if (R0 >= nrows) return;  // warp-uniform
  const bool has1 = R1 < nrows;
  double* row0 = S + (size_t)R0 * ld + o;
  double* row1 = S + (size_t)(has1 ? R1 : R0) * ld + o;
  constexpr int H = kTB / 32;  // entries per lane
  double a0[H], a1[H];
#pragma unroll
  for (int h = 0; h < H; ++h) {
    a0[h] = row0[lane + 32 * h];
    a1[h] = row1[lane + 32 * h];
  }
#pragma unroll
  for (int hj = 0; hj < H; ++hj)
#pragma unroll 8
    for (int jl = 0; jl < 32; ++jl) {
      const int j = 32 * hj + jl;
      const double x0 = __shfl_sync(0xffffffffu, a0[hj], jl);
      const double x1 = __shfl_sync(0xffffffffu, a1[hj], jl);
#pragma unroll
      for (int h = 0; h < H; ++h) {
        const int mrow = lane + 32 * h;
        if (mrow > j) {
          a0[h] = fma(-x0, Ls[mrow][j], a0[h]);
          a1[h] = fma(-x1, Ls[mrow][j], a1[h]);
        }
      }
    }
#pragma unroll
  for (int h = 0; h < H; ++h) {
    const double r = ri[lane + 32 * h];
    row0[lane + 32 * h] = a0[h] * r;
    if (has1) row1[lane + 32 * h] = a1[h] * r;
  }
}

// Strips of RH rows x 32 columns of the trailing lower triangle (column
// tiles [jlo, jhi) of 32 columns, every row from the tile's first down to the
// b row): S -= L_ik L_jk^T with panel k (in 32-column parts).  Each
// thread keeps RR x CC results in NA independent partial sums.
template <int RH>
__global__ void __launch_bounds__(128) k_tchol_update(double* S, int ld, int k, int nrows, int jlo, int jhi) {
  constexpr int RR = RH == 32 ? 2 : 1;
  constexpr int CC = RH / (4 * RR);
  constexpr int CG = kTC / CC;  // column groups
  constexpr int NA = RR * CC >= 8 ? 2 : 4;
  __shared__ double As[RH][kTC + 1];
  __shared__ double Bs[kTC][kTC + 1];
  int b = blockIdx.x, J = jlo;
  for (; J < jhi; ++J) {
    const int ns = (nrows - kTC * J + RH - 1) / RH;
    if (b < ns) break;
    b -= ns;
  }
  if (J >= jhi) return;
  const int row0 = kTC * J + b * RH, col0 = kTC * J;
  const int tid = threadIdx.x;
  const int rg = tid / CG, cg = tid % CG;
  double acc[NA][RR][CC];
#pragma unroll
  for (int h = 0; h < NA; ++h)
#pragma unroll
    for (int a = 0; a < RR; ++a)
#pragma unroll
      for (int c = 0; c < CC; ++c) acc[h][a][c] = 0.0;
  for (int half = 0; half < kTB / kTC; ++half) {
    const int o = k * kTB + half * kTC;
    if (half) __syncthreads();
    for (int idx = tid; idx < RH * kTC; idx += 128) {
      const int r = idx >> 5, c = idx & 31;
      As[r][c] = (row0 + r < nrows) ? S[(size_t)(row0 + r) * ld + o + c] : 0.0;
    }
    for (int idx = tid; idx < kTC * kTC; idx += 128) {
      const int r = idx >> 5, c = idx & 31;
      Bs[r][c] = S[(size_t)(col0 + r) * ld + o + c];
    }
    __syncthreads();
#pragma unroll 4
    for (int q0 = 0; q0 < kTC; q0 += NA) {
#pragma unroll
      for (int h = 0; h < NA; ++h) {
        const int q = q0 + h;
        double av[RR], bv[CC];
#pragma unroll
        for (int a = 0; a < RR; ++a) av[a] = As[rg * RR + a][q];
#pragma unroll
        for (int c = 0; c < CC; ++c) bv[c] = Bs[cg * CC + c][q];
#pragma unroll
        for (int a = 0; a < RR; ++a)
#pragma unroll
          for (int c = 0; c < CC; ++c) acc[h][a][c] = fma(av[a], bv[c], acc[h][a][c]);
      }
    }
  }
#pragma unroll
  for (int h = 1; h < NA; ++h)
#pragma unroll
    for (int a = 0; a < RR; ++a)
#pragma unroll
      for (int c = 0; c < CC; ++c) acc[0][a][c] += acc[h][a][c];
#pragma unroll
  for (int a = 0; a < RR; ++a) {
    const int r = row0 + rg * RR + a;
    if (r >= nrows) continue;
#pragma unroll
    for (int c = 0; c < CC; ++c) {
      const int col = col0 + cg * CC + c;
      if (col <= r) S[(size_t)r * ld + col] -= acc[0][a][c];
    }
  }
}

// Backward substitution, block row I (from the last): x_I = M_I^T (y_I - t_I)
// with y = the forward-substituted b row, then t_c += sum_r L[32 I + r][c] x_I[r]
// for every column c < 32 I (each column owned by one thread of one CTA).
__global__ void __launch_bounds__(256) k_tchol_bsolve(const double* __restrict__ S, double* ws, int ld, int n,
                                                       int I, double* x, const int* solve_ok) {
  __shared__ double us[kTB], xs[kTB];
  if (!*solve_ok) return;
  const int nt = ld / kTB, tid = threadIdx.x, o = I * kTB;
  double* t = ws + ws_t(nt);
  if (tid < kTB) us[tid] = S[(size_t)ld * ld + o + tid] - t[o + tid];
  __syncthreads();
  if (tid < kTB) {
    const double* M = ws + ws_M(nt, I);  // x_c = sum_{r >= c} M[r][c] u_r
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
#pragma unroll 4
    for (int r = 0; r < kTB; r += 4) {
      s0 = fma(M[r * kTB + tid], us[r], s0);
      s1 = fma(M[(r + 1) * kTB + tid], us[r + 1], s1);
      s2 = fma(M[(r + 2) * kTB + tid], us[r + 2], s2);
      s3 = fma(M[(r + 3) * kTB + tid], us[r + 3], s3);
    }
    const double xv = (s0 + s1) + (s2 + s3);
    xs[tid] = xv;
    if (blockIdx.x == 0 && o + tid < n) x[o + tid] = xv;
  }
  __syncthreads();
  const int c = blockIdx.x * blockDim.x + tid;
  if (c >= o) return;
  const double* Lr = S + (size_t)o * ld + c;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
#pragma unroll 4
  for (int r = 0; r < kTB; r += 4) {
    s0 = fma(Lr[(size_t)r * ld], xs[r], s0);
    s1 = fma(Lr[(size_t)(r + 1) * ld], xs[r + 1], s1);
    s2 = fma(Lr[(size_t)(r + 2) * ld], xs[r + 2], s2);
    s3 = fma(Lr[(size_t)(r + 3) * ld], xs[r + 3], s3);
  }
  t[c] += (s0 + s1) + (s2 + s3);
}

int update_blocks(int nrows, int jlo, int jhi, int rh) {
  int nb = 0;
  for (int J = jlo; J < jhi; ++J) nb += (nrows - kTC * J + rh - 1) / rh;
  return nb;
}

// Launch with a scheduling priority: the kernels on the factorisation's
// critical path take the device's greatest priority, the bulk trailing
// update its least, so free SM slots go to the critical path first.
template <typename... KArgs, typename... Args>
cudaError_t launch_prio(void (*kern)(KArgs...), int grid, int block, size_t smem, int prio, cudaStream_t st,
                        Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid, 1, 1);
  cfg.blockDim = dim3(block, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr;
  attr.id = cudaLaunchAttributePriority;
  attr.val.priority = prio;
  cfg.attrs = &attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}

}  // namespace

cudaError_t chol_tiled_setup(TiledChol* t) {
  if (t->side) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(k_tchol_tinv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTinvSmem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_tchol_trsm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrsmSmem);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&t->side, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&t->ev_panel, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&t->ev_rest, cudaEventDisableTiming);
  return e;
}

void chol_tiled_release(TiledChol* t) {
  if (t->side) {
    cudaStreamSynchronize(t->side);
    cudaStreamDestroy(t->side);
  }
  if (t->ev_panel) cudaEventDestroy(t->ev_panel);
  if (t->ev_rest) cudaEventDestroy(t->ev_rest);
  t->side = nullptr;
  t->ev_panel = t->ev_rest = nullptr;
}

int chol_tiled_stride(int n) { return ((n + kTB - 1) / kTB) * kTB; }

size_t chol_tiled_ws_doubles(int ld) { return ws_r(ld / kTB) + (size_t)ld; }

cudaError_t chol_tiled_launch(TiledChol& tc, double* S, double* ws, int ld, int n, double* x, int* solve_ok,
                              cudaStream_t st, long long* launches) {
  if (ld % kTB != 0 || ld < 2 * kTB) return cudaErrorInvalidValue;
  const int nt = ld / kTB, ntc = ld / kTC, nrows = ld + 1;  // b_schur is row ld
  const int per = kTB / kTC;  // column tiles per panel
  cudaStream_t sd = tc.side;
  long long nl = 0;
  int lo = 0, hi = 0;
  cudaDeviceGetStreamPriorityRange(&lo, &hi);  // lo: least, hi: greatest
  launch_prio(k_tchol_diag, 1, kDiagThreads, 0, hi, st, (const double*)S, ws, ld, 0, solve_ok);
  launch_prio(k_tchol_trsm, (nrows - kTB + 7) / 8, 128, kTrsmSmem, hi, st, S, (const double*)ws, ld, 0, nrows);
  nl += 2;
  for (int k = 0; k < nt; ++k) {
    // panel k is final
    bool rest = false;
    if (k + 2 < nt) {
      cudaEventRecord(tc.ev_panel, st);
      cudaStreamWaitEvent(sd, tc.ev_panel, 0);
      const int nb = update_blocks(nrows, per * (k + 2), ntc, 32);
      launch_prio(k_tchol_update<32>, nb, 128, 0, lo, sd, S, ld, k, nrows, per * (k + 2), ntc);
      cudaEventRecord(tc.ev_rest, sd);
      rest = true;
      ++nl;
    }
    if (k + 1 < nt) {
      const int nb = update_blocks(nrows, per * (k + 1), per * (k + 2), 8);
      launch_prio(k_tchol_update<8>, nb, 128, 0, hi, st, S, ld, k, nrows, per * (k + 1), per * (k + 2));
      launch_prio(k_tchol_diag, 1, kDiagThreads, 0, hi, st, (const double*)S, ws, ld, k + 1, solve_ok);
      const int below = nrows - (k + 2) * kTB;
      launch_prio(k_tchol_trsm, (below + 7) / 8, 128, kTrsmSmem, hi, st, S, (const double*)ws, ld, k + 1, nrows);
      nl += 3;
    }
    if (rest) cudaStreamWaitEvent(st, tc.ev_rest, 0);  // before those columns are touched
  }
  // backward substitution with the inverses of the diagonal tiles
  launch_prio(k_tchol_tinv, nt, kDiagThreads, kTinvSmem, hi, st, ws, ld);
  ++nl;
  cudaError_t e = cudaMemsetAsync(ws + ws_t(nt), 0, sizeof(double) * (size_t)ld, st);
  if (e != cudaSuccess) return e;
  for (int I = nt - 1; I >= 0; --I) {
    const int nb = I > 0 ? (I * kTB + 255) / 256 : 1;
    launch_prio(k_tchol_bsolve, nb, 256, 0, hi, st, (const double*)S, ws, ld, n, I, x, (const int*)solve_ok);
    ++nl;
  }
  if (launches) *launches += nl;
  return cudaGetLastError();
}

}  // namespace mcba
