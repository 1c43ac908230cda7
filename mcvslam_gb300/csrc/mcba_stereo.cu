// mcba_stereo.cu -- stereo matching of a rectified pair: descriptor search
// along the epipolar row band, 11 x 11 SAD refinement, parabola sub-pixel fit,
// median filter.
//
// Frame::ComputeStereoMatch (src/Frame.cpp:150-325) for a batch of frames:
//   k_rows    one CTA per frame: the row table (each right keypoint listed in
//             every row within 10 x mvScaleFactor[octave] of its y), as a CSR
//             of rows; list order is free because ranks are explicit below;
//   k_match   one half-warp per left keypoint: the candidates of its row
//             within one octave and inside [uL - maxD, uL - minD], Hamming
//             distances, the k = 2 match as the minimum of
//             (distance << 23 | right index) -- the reference's row lists are
//             in right-index order and keep the first of equal distances --
//             FilterRatio(0.70) and FilterThreshold(34); then lanes 0..10 each
//             take one row of the 11 x 11 patch at the keypoint's pyramid
//             level and accumulate the centre-subtracted absolute differences
//             for all 11 offsets, a shuffle reduction gives the 11 SADs, and
//             the first minimum, the parabola and the disparity test follow
//             in float exactly as the reference writes them;
//   k_median  one CTA per frame: the median of the frames' best SADs by a
//             two-pass 256-bin radix select, and the 0.4 / 1.6 x median
//             outlier rejection.
// The reference's undefined corners get a defined result (rows of a band
// outside the image dropped; a right window starting left of column 0 skips
// the keypoint, where OpenCV would throw; a frame with no matches skips the
// median filter).  Integer / gather work; no tensor cores by design.

#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <mutex>
#include <vector>

#include "mcba.h"

namespace {

constexpr int kHalf = 16;        // lanes per left keypoint
constexpr int kW = 5;            // patch half-width (w)
constexpr int kL = 5;            // offset half-range (L)
constexpr int kPatch = 2 * kW + 1;
constexpr int kOffs = 2 * kL + 1;
constexpr int kRightBits = 23;   // keys are distance << 23 | right index
constexpr int kMaxRight = 1 << kRightBits;
constexpr int kMaxRows = 8192;   // row-table rows (shared-memory counters)
constexpr unsigned kNoKey = 0xffffffffu;
constexpr float kRatio = 0.70f;  // FilterRatio(0.70), src/Frame.cpp:225
constexpr int kMaxDesc = 34;     // FilterThreshold(ORB_GOOD_THRESHOLD * 0.75) takes an int

__device__ __forceinline__ unsigned hamming32(const uint4& a0, const uint4& a1, const uint4& b0, const uint4& b1) {
  return __popc(a0.x ^ b0.x) + __popc(a0.y ^ b0.y) + __popc(a0.z ^ b0.z) + __popc(a0.w ^ b0.w) +
         __popc(a1.x ^ b1.x) + __popc(a1.y ^ b1.y) + __popc(a1.z ^ b1.z) + __popc(a1.w ^ b1.w);
}

// the row band of a right keypoint, clipped to the table
__device__ __forceinline__ void band(float y, float s, int rows, int* lo, int* hi) {
  const float r = __fmul_rn(10.f, s);
  *hi = min((int)ceilf(__fadd_rn(y, r)), rows - 1);
  *lo = max((int)floorf(__fsub_rn(y, r)), 0);
}

struct Work {
  int32_t* row_start;  // [F][rows + 1], frame-local offsets
  int32_t* row_kp;     // [n_right * max_band], frame f's lists at right_begin[f] * max_band
  int32_t* best;       // [n_left] best SAD of a kept match, -1 none
};

// One CTA per frame.
__global__ void __launch_bounds__(256) k_rows(mcba_stereo_batch B, int max_band, Work w) {
  extern __shared__ int cnt[];  // [rows + 1]
  const int f = blockIdx.x;
  const int rows = B.image_rows;
  const int r0 = B.right_begin[f], nr = B.right_begin[f + 1] - r0;
  for (int r = threadIdx.x; r <= rows; r += blockDim.x) cnt[r] = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < nr; i += blockDim.x) {
    int lo, hi;
    band(B.right_xy[2 * (size_t)(r0 + i) + 1], B.scale[B.right_oct[r0 + i]], rows, &lo, &hi);
    for (int y = lo; y <= hi; ++y) atomicAdd(&cnt[y], 1);
  }
  __syncthreads();
  // exclusive scan of rows + 1 counters: each thread a contiguous run
  __shared__ int tsum[256];
  const int per = (rows + 1 + blockDim.x - 1) / blockDim.x;
  const int a = threadIdx.x * per, e = min(rows + 1, a + per);
  int s = 0;
  for (int r = a; r < e; ++r) s += cnt[r];
  tsum[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int t = 0; t < (int)blockDim.x; ++t) {
      const int v = tsum[t];
      tsum[t] = run;
      run += v;
    }
  }
  __syncthreads();
  int32_t* rs = w.row_start + (size_t)f * (rows + 1);
  int run = tsum[threadIdx.x];
  for (int r = a; r < e; ++r) {
    const int v = cnt[r];
    rs[r] = run;
    cnt[r] = run;  // cursor
    run += v;
  }
  __syncthreads();
  int32_t* lists = w.row_kp + (size_t)r0 * max_band;
  for (int i = threadIdx.x; i < nr; i += blockDim.x) {
    int lo, hi;
    band(B.right_xy[2 * (size_t)(r0 + i) + 1], B.scale[B.right_oct[r0 + i]], rows, &lo, &hi);
    for (int y = lo; y <= hi; ++y) lists[atomicAdd(&cnt[y], 1)] = i;
  }
}

__device__ __forceinline__ int frame_of(const int32_t* begin, int n_frames, int i) {
  int lo = 0, hi = n_frames - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (begin[mid] <= i) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__global__ void __launch_bounds__(128) k_match(mcba_stereo_batch B, int n_left, int max_band, Work w,
                                               float* __restrict__ u_right, float* __restrict__ depth) {
  const int lane = threadIdx.x & 31;
  const int hl = lane & (kHalf - 1);
  const unsigned hmask = 0xffffu << (lane & 16);
  const int iL = (blockIdx.x * blockDim.x + threadIdx.x) / kHalf;
  if (iL >= n_left) return;  // whole half-warps leave together
  const int f = frame_of(B.left_begin, B.n_frames, iL);
  const int l0 = B.left_begin[f];
  const int r0 = B.right_begin[f];
  const int rows = B.image_rows;
  const int levelL = B.left_oct[iL];
  const float uL = B.left_xy[2 * (size_t)iL], vL = B.left_xy[2 * (size_t)iL + 1];
  float out_u = -1.f, out_d = -1.f;
  int out_best = -1;
  const float minD = 1.f;
  const float maxD = fminf(__fdiv_rn(B.bf, B.b), 1000.f);
  const float minU = __fsub_rn(uL, maxD), maxU = __fsub_rn(uL, minD);
  bool go = vL >= 0.f && vL < (float)rows && !(maxU < 0.f) && levelL >= 0 && levelL < B.n_levels;
  unsigned b0 = kNoKey, b1 = kNoKey;
  if (go) {
    const int row = (int)vL;
    const int32_t* rs = w.row_start + (size_t)f * (rows + 1);
    const int32_t* lists = w.row_kp + (size_t)r0 * max_band;
    const uint4* ld = reinterpret_cast<const uint4*>(B.left_desc);
    const uint4* rd = reinterpret_cast<const uint4*>(B.right_desc);
    const uint4 q0 = ld[2 * (size_t)iL], q1 = ld[2 * (size_t)iL + 1];
    const int e = rs[row + 1];
    for (int p = rs[row] + hl; p < e; p += kHalf) {
      const int iR = lists[p];
      const int o = B.right_oct[r0 + iR];
      if (o < levelL - 1 || o > levelL + 1) continue;
      const float uR = B.right_xy[2 * (size_t)(r0 + iR)];
      if (!(uR >= minU && uR <= maxU)) continue;
      const unsigned key =
          (hamming32(q0, q1, rd[2 * (size_t)(r0 + iR)], rd[2 * (size_t)(r0 + iR) + 1]) << kRightBits) | (unsigned)iR;
      const unsigned hi2 = max(key, b0);
      b0 = min(key, b0);
      b1 = min(hi2, b1);
    }
  }
#pragma unroll
  for (int d = 1; d < kHalf; d <<= 1) {
    const unsigned c0 = __shfl_xor_sync(hmask, b0, d, kHalf);
    const unsigned c1 = __shfl_xor_sync(hmask, b1, d, kHalf);
    const unsigned hi0 = max(b0, c0);
    b0 = min(b0, c0);
    b1 = min(hi0, min(b1, c1));
  }
  // KnnMatch k = 2, FilterRatio(0.70), FilterThreshold(34) -- uniform in the half-warp
  if (b0 != kNoKey) {
    const unsigned d0 = b0 >> kRightBits;
    const unsigned d1 = b1 != kNoKey ? (b1 >> kRightBits) : 999u;
    go = (float)d0 / (float)d1 <= kRatio && !((float)d0 > (float)kMaxDesc);
  } else {
    go = false;
  }
  float scaleduR0 = 0.f;
  int yv = 0, xl = 0, xr = 0, colsL = 0;
  const uint8_t* imL = nullptr;
  const uint8_t* imR = nullptr;
  if (go) {
    const int iR = (int)(b0 & (kMaxRight - 1));
    const float uR0 = B.right_xy[2 * (size_t)(r0 + iR)];
    const float sf = B.inv_scale[levelL];
    const float scaleduL = roundf(__fmul_rn(uL, sf));
    const float scaledvL = roundf(__fmul_rn(vL, sf));
    scaleduR0 = roundf(__fmul_rn(uR0, sf));
    const int rowsL = B.level_rows[levelL];
    colsL = B.level_cols[levelL];
    if (scaledvL - kW < 0 || scaledvL + kW + 1 >= rowsL || scaleduL - kW < 0 || scaleduL + kW + 1 >= colsL) go = false;
    const float iniu = __fsub_rn(__fadd_rn(scaleduR0, (float)kL), (float)kW);
    const float endu = __fadd_rn(__fadd_rn(__fadd_rn(scaleduR0, (float)kL), (float)kW), 1.f);
    if (iniu < 0 || endu >= colsL) go = false;
    yv = (int)scaledvL;
    xl = (int)scaleduL;
    xr = (int)scaleduR0;
    if (xr - kL - kW < 0) go = false;  // the reference's colRange would throw
    imL = B.left_pyr + (size_t)f * B.pyr_bytes + B.level_offset[levelL];
    imR = B.right_pyr + (size_t)f * B.pyr_bytes + B.level_offset[levelL];
  }
  if (go) {  // uniform in the half-warp
    // lane hl < 11 takes patch row hl: 11 left pixels, 21 right pixels
    int Lp[kPatch], Rp[kPatch + 2 * kL];
    const int rr = min(hl, kPatch - 1);
    const uint8_t* lrow = imL + (size_t)(yv - kW + rr) * colsL + (xl - kW);
    const uint8_t* rrow = imR + (size_t)(yv - kW + rr) * colsL + (xr - kL - kW);
#pragma unroll
    for (int c = 0; c < kPatch; ++c) Lp[c] = lrow[c];
#pragma unroll
    for (int c = 0; c < kPatch + 2 * kL; ++c) Rp[c] = rrow[c];
    // centres: the left patch's and each right window's (patch row kW)
    const int base = lane & 16;
    const int cL = __shfl_sync(hmask, Lp[kW], base + kW);
    int sad[kOffs];
#pragma unroll
    for (int k = 0; k < kOffs; ++k) {
      const int cR = __shfl_sync(hmask, Rp[k + kW], base + kW);
      int acc = 0;
#pragma unroll
      for (int c = 0; c < kPatch; ++c) acc += abs((Lp[c] - cL) - (Rp[k + c] - cR));
      sad[k] = hl < kPatch ? acc : 0;
    }
#pragma unroll
    for (int k = 0; k < kOffs; ++k)
#pragma unroll
      for (int d = 1; d < kHalf; d <<= 1) sad[k] += __shfl_xor_sync(hmask, sad[k], d, kHalf);
    int bestDist = INT_MAX, bestinc = 0;
#pragma unroll
    for (int k = 0; k < kOffs; ++k)
      if (sad[k] < bestDist) {
        bestDist = sad[k];
        bestinc = k - kL;
      }
    if (bestinc != -kL && bestinc != kL) {
      float d1 = 0.f, d2 = 0.f, d3 = 0.f;
#pragma unroll
      for (int k = 1; k < kOffs - 1; ++k)
        if (k - kL == bestinc) {
          d1 = (float)sad[k - 1];
          d2 = (float)sad[k];
          d3 = (float)sad[k + 1];
        }
      const float deltaR =
          __fdiv_rn(__fsub_rn(d1, d3), __fmul_rn(2.0f, __fsub_rn(__fadd_rn(d1, d3), __fmul_rn(2.0f, d2))));
      if (!(deltaR < -1 || deltaR > 1)) {
        const float bestuR =
            __fmul_rn(B.scale[levelL], __fadd_rn(__fadd_rn(scaleduR0, (float)bestinc), deltaR));
        const float disparity = __fsub_rn(uL, bestuR);
        if (disparity >= minD && disparity < maxD) {
          out_u = bestuR;
          out_d = __fdiv_rn(B.bf, disparity);
          out_best = bestDist;
        }
      }
    }
  }
  if (hl == 0) {
    u_right[iL] = out_u;
    depth[iL] = out_d;
    w.best[iL] = out_best;
  }
  (void)l0;
}

// One CTA per frame: the median of the kept best SADs (the (n/2)-th smallest,
// n the number kept), then the 1.6 x / 0.4 x median rejection.
__global__ void __launch_bounds__(256) k_median(mcba_stereo_batch B, Work w, float* __restrict__ u_right,
                                                float* __restrict__ depth) {
  __shared__ int hist[256];
  __shared__ int sel[3];  // count, high byte, target rank
  const int f = blockIdx.x;
  const int l0 = B.left_begin[f], nl = B.left_begin[f + 1] - l0;
  for (int t = threadIdx.x; t < 256; t += blockDim.x) hist[t] = 0;
  if (threadIdx.x == 0) sel[0] = 0;
  __syncthreads();
  // SADs are at most 121 x 510 < 2^16: two byte digits
  for (int i = threadIdx.x; i < nl; i += blockDim.x) {
    const int v = w.best[l0 + i];
    if (v >= 0) {
      atomicAdd(&hist[(v >> 8) & 255], 1);
      atomicAdd(&sel[0], 1);
    }
  }
  __syncthreads();
  const int n = sel[0];
  if (n == 0) return;
  if (threadIdx.x == 0) {
    int k = n / 2, run = 0, bin = 0;
    for (; bin < 256; ++bin) {
      if (run + hist[bin] > k) break;
      run += hist[bin];
    }
    sel[1] = bin;
    sel[2] = k - run;
  }
  __syncthreads();
  const int hi = sel[1];
  for (int t = threadIdx.x; t < 256; t += blockDim.x) hist[t] = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < nl; i += blockDim.x) {
    const int v = w.best[l0 + i];
    if (v >= 0 && ((v >> 8) & 255) == hi) atomicAdd(&hist[v & 255], 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int k = sel[2], run = 0, bin = 0;
    for (; bin < 256; ++bin) {
      if (run + hist[bin] > k) break;
      run += hist[bin];
    }
    sel[1] = (hi << 8) | bin;
  }
  __syncthreads();
  const float median = (float)sel[1];
  const float th_max = __fmul_rn(1.6f, median);
  const float th_min = __double2float_rn(__dmul_rn(0.4, (double)median));
  for (int i = threadIdx.x; i < nl; i += blockDim.x) {
    const int v = w.best[l0 + i];
    if (v >= 0 && ((float)v > th_max || (float)v < th_min)) {
      u_right[l0 + i] = -1.f;
      depth[l0 + i] = -1.f;
    }
  }
}

struct Scratch {
  std::mutex mu;
  std::vector<void*> ptr;
  std::vector<size_t> cap;
};
Scratch g_scratch;

cudaError_t scratch(int dev, size_t bytes, void** out) {
  std::lock_guard<std::mutex> lk(g_scratch.mu);
  if ((int)g_scratch.ptr.size() <= dev) {
    g_scratch.ptr.resize(dev + 1, nullptr);
    g_scratch.cap.resize(dev + 1, 0);
  }
  if (g_scratch.cap[dev] < bytes) {
    if (g_scratch.ptr[dev]) cudaFree(g_scratch.ptr[dev]);
    g_scratch.ptr[dev] = nullptr;
    g_scratch.cap[dev] = 0;
    const cudaError_t e = cudaMalloc(&g_scratch.ptr[dev], bytes);
    if (e != cudaSuccess) return e;
    g_scratch.cap[dev] = bytes;
  }
  *out = g_scratch.ptr[dev];
  return cudaSuccess;
}

size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

// the widest row band any right keypoint can have
int max_band(const mcba_stereo_batch* b) {
  float s = 0.f;
  for (int l = 0; l < b->n_levels; ++l) s = std::max(s, b->scale[l]);
  return 2 * (int)std::ceil(10.f * s) + 3;
}

size_t scratch_bytes(const mcba_stereo_batch* b, int n_left, int n_right) {
  return align16((size_t)b->n_frames * (b->image_rows + 1) * 4) +
         align16((size_t)n_right * max_band(b) * 4) + align16((size_t)n_left * 4);
}

Work carve(void* base, const mcba_stereo_batch* b, int n_left, int n_right) {
  char* p = static_cast<char*>(base);
  Work w;
  w.row_start = reinterpret_cast<int32_t*>(p);
  p += align16((size_t)b->n_frames * (b->image_rows + 1) * 4);
  w.row_kp = reinterpret_cast<int32_t*>(p);
  p += align16((size_t)n_right * max_band(b) * 4);
  w.best = reinterpret_cast<int32_t*>(p);
  return w;
}

// host-side checks of what the kernels rely on (sizes and tables only)
int check_tables(const mcba_stereo_batch* b) {
  if (b->n_frames < 0 || b->n_levels <= 0 || b->n_levels > MCBA_MAX_LEVELS) return MCBA_ERR_INVALID;
  if (b->image_rows <= 0) return MCBA_ERR_INVALID;
  if (b->image_rows > kMaxRows) return MCBA_ERR_TOO_LARGE;
  if (!(b->b > 0.f) || !std::isfinite(b->bf)) return MCBA_ERR_INVALID;
  for (int l = 0; l < b->n_levels; ++l) {
    if (!(b->scale[l] > 0.f) || !std::isfinite(b->scale[l]) || !std::isfinite(b->inv_scale[l])) return MCBA_ERR_INVALID;
    if (b->scale[l] > 1000.f) return MCBA_ERR_TOO_LARGE;
    if (b->level_rows[l] <= 0 || b->level_cols[l] <= 0 || b->level_offset[l] < 0) return MCBA_ERR_INVALID;
    if (b->level_offset[l] + (int64_t)b->level_rows[l] * b->level_cols[l] > b->pyr_bytes) return MCBA_ERR_INVALID;
  }
  return MCBA_OK;
}

int launch(const mcba_stereo_batch* b, int n_left, int n_right, float* u_right, float* depth, void* work,
           cudaStream_t st) {
  const Work w = carve(work, b, n_left, n_right);
  const int mb = max_band(b);
  k_rows<<<b->n_frames, 256, (size_t)(b->image_rows + 1) * sizeof(int), st>>>(*b, mb, w);
  if (n_left > 0) {
    const long long threads = (long long)n_left * kHalf;
    k_match<<<(unsigned)((threads + 127) / 128), 128, 0, st>>>(*b, n_left, mb, w, u_right, depth);
  }
  k_median<<<b->n_frames, 256, 0, st>>>(*b, w, u_right, depth);
  return cudaGetLastError() == cudaSuccess ? MCBA_OK : MCBA_ERR_CUDA;
}

bool aligned(const void* p, uintptr_t a) { return (reinterpret_cast<uintptr_t>(p) & (a - 1)) == 0; }

}  // namespace

extern "C" int mcba_stereo_match_device(const mcba_stereo_batch* b, int32_t n_left, int32_t n_right,
                                        float* u_right, float* depth, void* stream) {
  if (!b || n_left < 0 || n_right < 0) return MCBA_ERR_INVALID;
  const int t = check_tables(b);
  if (t) return t;
  if (b->n_frames == 0) return MCBA_OK;
  if (!b->left_begin || !b->right_begin || !b->left_pyr || !b->right_pyr) return MCBA_ERR_INVALID;
  if (n_left > 0 && (!b->left_xy || !b->left_oct || !b->left_desc || !u_right || !depth ||
                     !aligned(b->left_desc, 16) || !aligned(b->left_xy, 8)))
    return MCBA_ERR_INVALID;
  if (n_right > 0 && (!b->right_xy || !b->right_oct || !b->right_desc || !aligned(b->right_desc, 16)))
    return MCBA_ERR_INVALID;
  if ((long long)n_right * max_band(b) >= (1ll << 31)) return MCBA_ERR_TOO_LARGE;
  int dev = 0;
  cudaGetDevice(&dev);
  void* work = nullptr;
  if (scratch(dev, scratch_bytes(b, n_left, n_right), &work) != cudaSuccess) return MCBA_ERR_NOMEM;
  return launch(b, n_left, n_right, u_right, depth, work, static_cast<cudaStream_t>(stream));
}

extern "C" int mcba_stereo_match(int32_t device, const mcba_stereo_batch* b, float* u_right, float* depth,
                                 double* ms_device) {
  if (!b) return MCBA_ERR_INVALID;
  const int t = check_tables(b);
  if (t) return t;
  if (ms_device) *ms_device = 0.0;
  const int F = b->n_frames;
  if (F == 0) return MCBA_OK;
  if (!b->left_begin || !b->right_begin || !b->left_pyr || !b->right_pyr) return MCBA_ERR_INVALID;
  if (b->left_begin[0] != 0 || b->right_begin[0] != 0) return MCBA_ERR_INVALID;
  for (int f = 0; f < F; ++f) {
    if (b->left_begin[f + 1] < b->left_begin[f] || b->right_begin[f + 1] < b->right_begin[f]) return MCBA_ERR_INVALID;
    if (b->right_begin[f + 1] - b->right_begin[f] >= kMaxRight) return MCBA_ERR_TOO_LARGE;
  }
  const int n_left = b->left_begin[F], n_right = b->right_begin[F];
  if (n_left > 0 && (!b->left_xy || !b->left_oct || !b->left_desc || !u_right || !depth)) return MCBA_ERR_INVALID;
  if (n_right > 0 && (!b->right_xy || !b->right_oct || !b->right_desc)) return MCBA_ERR_INVALID;
  for (int i = 0; i < n_left; ++i) {
    if (b->left_oct[i] < 0 || b->left_oct[i] >= b->n_levels) return MCBA_ERR_INVALID;
    if (!std::isfinite(b->left_xy[2 * (size_t)i]) || !std::isfinite(b->left_xy[2 * (size_t)i + 1]))
      return MCBA_ERR_NONFINITE;
  }
  for (int i = 0; i < n_right; ++i) {
    if (b->right_oct[i] < 0 || b->right_oct[i] >= b->n_levels) return MCBA_ERR_INVALID;
    if (!std::isfinite(b->right_xy[2 * (size_t)i]) || !std::isfinite(b->right_xy[2 * (size_t)i + 1]))
      return MCBA_ERR_NONFINITE;
  }
  if ((long long)n_right * max_band(b) >= (1ll << 31)) return MCBA_ERR_TOO_LARGE;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return MCBA_ERR_NO_DEVICE;
  if (device < 0 || device >= n || cudaSetDevice(device) != cudaSuccess) return MCBA_ERR_INVALID;

  struct Part {
    const void* src;
    size_t bytes;
    size_t off;
  };
  const size_t pyr = (size_t)F * (size_t)b->pyr_bytes;
  std::vector<Part> parts = {
      {b->left_pyr, pyr, 0},                         {b->right_pyr, pyr, 0},
      {b->left_begin, 4 * (size_t)(F + 1), 0},       {b->left_xy, 8 * (size_t)n_left, 0},
      {b->left_oct, 4 * (size_t)n_left, 0},          {b->left_desc, 32 * (size_t)n_left, 0},
      {b->right_begin, 4 * (size_t)(F + 1), 0},      {b->right_xy, 8 * (size_t)n_right, 0},
      {b->right_oct, 4 * (size_t)n_right, 0},        {b->right_desc, 32 * (size_t)n_right, 0},
      {nullptr, 4 * (size_t)n_left, 0},              {nullptr, 4 * (size_t)n_left, 0},
      {nullptr, scratch_bytes(b, n_left, n_right), 0}};
  size_t total = 0;
  for (Part& p : parts) {
    p.off = total;
    total += align16(p.bytes);
  }
  char* dbase = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int r = MCBA_ERR_CUDA;
  do {
    if (cudaMalloc(&dbase, std::max<size_t>(total, 16)) != cudaSuccess) {
      r = MCBA_ERR_NOMEM;
      break;
    }
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) break;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    bool ok = true;
    for (const Part& p : parts)
      if (p.src && p.bytes && cudaMemcpyAsync(dbase + p.off, p.src, p.bytes, cudaMemcpyHostToDevice, st) != cudaSuccess)
        ok = false;
    if (!ok) break;
    auto at = [&](int i) { return static_cast<void*>(dbase + parts[i].off); };
    mcba_stereo_batch d = *b;
    d.left_pyr = static_cast<const uint8_t*>(at(0));
    d.right_pyr = static_cast<const uint8_t*>(at(1));
    d.left_begin = static_cast<const int32_t*>(at(2));
    d.left_xy = static_cast<const float*>(at(3));
    d.left_oct = static_cast<const int32_t*>(at(4));
    d.left_desc = static_cast<const uint8_t*>(at(5));
    d.right_begin = static_cast<const int32_t*>(at(6));
    d.right_xy = static_cast<const float*>(at(7));
    d.right_oct = static_cast<const int32_t*>(at(8));
    d.right_desc = static_cast<const uint8_t*>(at(9));
    float* du = static_cast<float*>(at(10));
    float* dd = static_cast<float*>(at(11));
    cudaEventRecord(e0, st);
    r = launch(&d, n_left, n_right, du, dd, at(12), st);
    cudaEventRecord(e1, st);
    if (r) break;
    r = MCBA_ERR_CUDA;
    if (n_left && cudaMemcpyAsync(u_right, du, 4 * (size_t)n_left, cudaMemcpyDeviceToHost, st) != cudaSuccess) break;
    if (n_left && cudaMemcpyAsync(depth, dd, 4 * (size_t)n_left, cudaMemcpyDeviceToHost, st) != cudaSuccess) break;
    if (cudaStreamSynchronize(st) != cudaSuccess) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms_device) *ms_device = ms;
    r = MCBA_OK;
  } while (false);
  if (st) cudaStreamSynchronize(st);
  cudaFree(dbase);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  return r;
}
