// mcba_project.cu -- map-point projection + windowed descriptor match.
//
// Object::ProjectBunchMapPoints (src/Object.cpp:208-236) for a batch of
// objects (one camera of one frame each), every map point of every object in
// one launch:
//   k_grid     one CTA per object: the 30 x 30 keypoint grid of
//              Object::AssignFeaturesToGrid / PosInGrid (src/Object.cpp:182-201,
//              250-257) as a stable CSR (cells in x-major order, keypoints in
//              index order within a cell), plus copies of the keypoint
//              positions and descriptors in CSR order so the search below
//              reads them contiguously; resets the claim slots and counts;
//   k_project  one warp per 32 map points.  Each lane projects one map point:
//              Pc = R X + t (float products summed in double, one rounding --
//              how OpenCV evaluates `R * X + t` on CV_32F), Pinhole::project
//              in float, r = r_threshold x mvScaleFactor[level] and the cell
//              rectangle of GetFeaturesInArea (src/Object.cpp:263-300).  Then
//              groups of 8 lanes take the map points in turn: a cell row of
//              the rectangle is one contiguous CSR range, the 8 lanes stride
//              over it, test the window, take Hamming distances to the map
//              point's descriptor and keep a top-2, merged across the group
//              with three shuffles; FilterRatio / FilterThreshold as at
//              src/Object.cpp:226;
//   k_bind     one thread per keypoint: the bindings AddMapPoint
//              (src/Object.cpp:113-137) leaves after the whole visit.
//
// Order independence.  The reference visits candidates cell by cell (x
// outer, y inner) and within a cell in keypoint order, keeping the first of
// equal distances.  That visit order is exactly the order of positions in the
// stable CSR, so the match is the minimum of the 64-bit key
// (distance << 32 | CSR position), whatever lane finds it.  AddMapPoint's
// effect after visiting map points m = 0, 1, ... in order is: a keypoint
// claimed in this call is bound to its LAST claimant (atomicMax over the
// visit position), and a keypoint that is not claimed loses its old binding
// exactly when that map point matched elsewhere in this call (DelMapPoint on
// the map point); the caller passes that old binding as mp_prev_kp.
// Integer / latency-bound gather work; no tensor cores by design.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <mutex>
#include <vector>

#include "mcba.h"

namespace {

constexpr int kGridCols = 30;  // FRAME_GRID_COLS (include/Object.hpp:28)
constexpr int kGridRows = 30;  // FRAME_GRID_ROWS (include/Object.hpp:27)
constexpr int kCells = kGridCols * kGridRows;
constexpr int kCellStride = kCells + 1;
constexpr int kGroup = 8;  // lanes per map point in the search
constexpr unsigned kNoKey = 0xffffffffu;
constexpr int kPosBits = 23;  // keys are distance << 23 | CSR position
constexpr int kMaxObjectKps = 1 << kPosBits;

__device__ __forceinline__ unsigned hamming32(const uint4& a0, const uint4& a1, const uint4& b0, const uint4& b1) {
  return __popc(a0.x ^ b0.x) + __popc(a0.y ^ b0.y) + __popc(a0.z ^ b0.z) + __popc(a0.w ^ b0.w) +
         __popc(a1.x ^ b1.x) + __popc(a1.y ^ b1.y) + __popc(a1.z ^ b1.z) + __popc(a1.w ^ b1.w);
}

// PosInGrid: round((x - 0) * 30 / cols) in double; -1 outside the grid
__device__ __forceinline__ int grid_cell(float x, float y, double inv_w, double inv_h) {
  const double gx = round((double)x * inv_w);
  const double gy = round((double)y * inv_h);
  if (!(gx >= 0.0 && gx < (double)kGridCols && gy >= 0.0 && gy < (double)kGridRows)) return -1;
  return (int)gx * kGridRows + (int)gy;
}

struct Work {
  int32_t* cell_start;  // [O][901] CSR offsets, object-local
  int32_t* cell_kp;     // [n_kp] CSR position -> object-local keypoint
  float2* xy_csr;       // [n_kp] keypoint position in CSR order
  uint4* desc_csr;      // [n_kp][2] descriptor in CSR order
  double* obj_d;        // [O][16] R (9), t (3) in double, 30 / cols, 30 / rows
  int32_t* claim;       // [n_kp] last claimant (object-local map point) or -1
  uint8_t* cleared;     // [n_kp] old binding removed by DelMapPoint(map point)
};

// One CTA per object.  Cell counts and an exclusive scan give the CSR
// offsets; then, segment by segment, each of the 8 warps ranks a contiguous
// slice of the keypoints (per-warp cell counts, prefixed across warps per
// cell, then __match_any_sync ranks inside 32-keypoint chunks), which places
// every keypoint after all keypoints of lower index in its cell -- a stable
// counting sort.  Finally the CTA gathers the CSR-order copies.
constexpr int kSeg = 4096;  // keypoints ranked per segment
constexpr int kWarpsGrid = 8;

__global__ void __launch_bounds__(256) k_grid(const int32_t* __restrict__ kp_begin, const float* __restrict__ kp_xy,
                                              const uint4* __restrict__ kp_desc, const int32_t* __restrict__ obj_size,
                                              const float* __restrict__ obj_Rt, Work w,
                                              int32_t* __restrict__ obj_count) {
  __shared__ int cursor[kCells];
  __shared__ int hist[kWarpsGrid][kCells];
  __shared__ short kc[kSeg];
  __shared__ int wsum[kWarpsGrid];
  const int o = blockIdx.x;
  const int k0 = kp_begin[o], nk = kp_begin[o + 1] - k0;
  const double inv_w = (double)kGridCols / (double)obj_size[2 * o];
  const double inv_h = (double)kGridRows / (double)obj_size[2 * o + 1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int c = threadIdx.x; c < kCells; c += blockDim.x) cursor[c] = 0;
  if (threadIdx.x == 0) obj_count[o] = 0;
  if (threadIdx.x < 12) w.obj_d[16 * o + threadIdx.x] = (double)obj_Rt[12 * o + threadIdx.x];
  if (threadIdx.x == 12) w.obj_d[16 * o + 12] = inv_w;
  if (threadIdx.x == 13) w.obj_d[16 * o + 13] = inv_h;
  __syncthreads();
  for (int i = threadIdx.x; i < nk; i += blockDim.x) {
    w.claim[k0 + i] = -1;
    w.cleared[k0 + i] = 0;
  }
  if (nk >= kMaxObjectKps) {
    // CSR positions would not fit the 23-bit key field: an empty grid, so
    // the object's map points match nothing (the host entry rejects it)
    if (threadIdx.x == 0) {
      int32_t* cs0 = w.cell_start + (size_t)o * kCellStride;
      for (int c = 0; c <= kCells; ++c) cs0[c] = 0;
    }
    return;
  }
  for (int i = threadIdx.x; i < nk; i += blockDim.x) {
    const int c = grid_cell(kp_xy[2 * (size_t)(k0 + i)], kp_xy[2 * (size_t)(k0 + i) + 1], inv_w, inv_h);
    if (c >= 0) atomicAdd(&cursor[c], 1);
  }
  __syncthreads();
  // exclusive scan of 900 counts: 256 threads x 4 consecutive cells
  int v[4], s = 0;
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int c = 4 * threadIdx.x + e;
    v[e] = c < kCells ? cursor[c] : 0;
    s += v[e];
  }
  int incl = s;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int n = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += n;
  }
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  int run = incl - s;
  for (int q = 0; q < warp; ++q) run += wsum[q];
  int32_t* cs = w.cell_start + (size_t)o * kCellStride;
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int c = 4 * threadIdx.x + e;
    if (c < kCells) {
      cs[c] = run;
      cursor[c] = run;  // becomes the cell's cursor
    }
    run += v[e];
  }
  if (threadIdx.x == blockDim.x - 1) cs[kCells] = run;
  for (int seg = 0; seg < nk; seg += kSeg) {
    const int len = min(kSeg, nk - seg);
    const int slice = (len + kWarpsGrid - 1) / kWarpsGrid;
    __syncthreads();  // cursors of the previous segment are final
    for (int j = threadIdx.x; j < len; j += blockDim.x)
      kc[j] = (short)grid_cell(kp_xy[2 * (size_t)(k0 + seg + j)], kp_xy[2 * (size_t)(k0 + seg + j) + 1], inv_w,
                               inv_h);
    for (int c = threadIdx.x; c < kWarpsGrid * kCells; c += blockDim.x) (&hist[0][0])[c] = 0;
    __syncthreads();
    const int j0 = warp * slice, j1 = min(len, j0 + slice);
    for (int j = j0 + lane; j < j1; j += 32)
      if (kc[j] >= 0) atomicAdd(&hist[warp][kc[j]], 1);
    __syncthreads();
    for (int c = threadIdx.x; c < kCells; c += blockDim.x) {
      int r = cursor[c];
#pragma unroll
      for (int q = 0; q < kWarpsGrid; ++q) {
        const int t = hist[q][c];
        hist[q][c] = r;  // becomes warp q's cursor for cell c
        r += t;
      }
      cursor[c] = r;
    }
    __syncthreads();
    for (int base = j0; base < j1; base += 32) {
      const int j = base + lane;
      const int c = j < j1 ? (int)kc[j] : -1;
      const unsigned peers = __match_any_sync(0xffffffffu, c);
      const int rank = __popc(peers & ((1u << lane) - 1u));
      const int pos = c >= 0 ? hist[warp][c] + rank : 0;
      __syncwarp();
      if (c >= 0) {
        w.cell_kp[k0 + pos] = seg + j;
        if (lane == __ffs(peers) - 1) hist[warp][c] += __popc(peers);
      }
      __syncwarp();
    }
  }
  __syncthreads();
  const int n_grid = cs[kCells];
  for (int p = threadIdx.x; p < n_grid; p += blockDim.x) {
    const int i = w.cell_kp[k0 + p];
    w.xy_csr[k0 + p] = reinterpret_cast<const float2*>(kp_xy)[k0 + i];
    w.desc_csr[2 * (size_t)(k0 + p)] = kp_desc[2 * (size_t)(k0 + i)];
    w.desc_csr[2 * (size_t)(k0 + p) + 1] = kp_desc[2 * (size_t)(k0 + i) + 1];
  }
}

__global__ void __launch_bounds__(128) k_project(
    int n_objects, int n_mp, const int32_t* __restrict__ mp_begin, const float* __restrict__ obj_Rt,
    const float* __restrict__ obj_K, const int32_t* __restrict__ obj_size, const float* __restrict__ obj_radius,
    const float* __restrict__ obj_scale, int n_levels, float ratio, int max_dist, const int32_t* __restrict__ kp_begin,
    const float* __restrict__ mp_X, const uint4* __restrict__ mp_desc, const int32_t* __restrict__ mp_level,
    const int32_t* __restrict__ mp_prev_kp, Work w, int32_t* __restrict__ mp_match, int32_t* __restrict__ obj_count) {
  const int lane = threadIdx.x & 31;
  const int m = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32 + lane;
  // ---- per lane: project one map point
  int o = 0, minx = 0, maxx = -1, miny = 0, maxy = -1;
  float u = 0.f, v = 0.f, rad = 0.f;
  if (m < n_mp) {
    int lo = 0, hi = n_objects - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (mp_begin[mid] <= m) lo = mid; else hi = mid - 1;
    }
    o = lo;
    const int level = mp_level[m];
    if (level >= 0 && level < n_levels) {
      const double* Rt = w.obj_d + 16 * (size_t)o;
      const double X0 = mp_X[3 * (size_t)m], X1 = mp_X[3 * (size_t)m + 1], X2 = mp_X[3 * (size_t)m + 2];
      float Pc[3];
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        // products of floats are exact in double, so the sum is rounded the
        // same with or without contraction
        double s = Rt[3 * r] * X0;
        s += Rt[3 * r + 1] * X1;
        s += Rt[3 * r + 2] * X2;
        Pc[r] = (float)(s + Rt[9 + r]);
      }
      if (!(Pc[2] < 0.f)) {
        const float fx = obj_K[4 * o], fy = obj_K[4 * o + 1], cx = obj_K[4 * o + 2], cy = obj_K[4 * o + 3];
        u = __fadd_rn(__fdiv_rn(__fmul_rn(fx, Pc[0]), Pc[2]), cx);
        v = __fadd_rn(__fdiv_rn(__fmul_rn(fy, Pc[1]), Pc[2]), cy);
        rad = __fmul_rn(obj_radius[o], obj_scale[(size_t)o * n_levels + level]);
        // GetFeaturesInArea rejects u, v outside [0, cols) x [0, rows); NaN has no cells
        if (u >= 0.f && v >= 0.f && u < (float)obj_size[2 * o] && v < (float)obj_size[2 * o + 1]) {
          const double inv_w = w.obj_d[16 * o + 12], inv_h = w.obj_d[16 * o + 13];
          minx = max(0, (int)floor((double)__fsub_rn(u, rad) * inv_w));
          maxx = min(kGridCols - 1, (int)ceil((double)__fadd_rn(u, rad) * inv_w));
          miny = max(0, (int)floor((double)__fsub_rn(v, rad) * inv_h));
          maxy = min(kGridRows - 1, (int)ceil((double)__fadd_rn(v, rad) * inv_h));
        }
      }
    }
  }
  // ---- groups of 8 lanes search for the warp's 32 map points, 4 at a time
  const int g = lane >> 3, gl = lane & (kGroup - 1);
  for (int round = 0; round < 32 / 4; ++round) {
    const int src = round * 4 + g;
    const int mm = __shfl_sync(0xffffffffu, m, src);
    const int oo = __shfl_sync(0xffffffffu, o, src);
    const float uu = __shfl_sync(0xffffffffu, u, src);
    const float vv = __shfl_sync(0xffffffffu, v, src);
    const float rr = __shfl_sync(0xffffffffu, rad, src);
    const int x0 = __shfl_sync(0xffffffffu, minx, src);
    const int x1 = __shfl_sync(0xffffffffu, maxx, src);
    const int y0 = __shfl_sync(0xffffffffu, miny, src);
    const int y1 = __shfl_sync(0xffffffffu, maxy, src);
    unsigned b0 = kNoKey, b1 = kNoKey;
    int k0 = 0;
    if (mm < n_mp && x0 <= x1 && y0 <= y1) {  // uniform within the group
      k0 = kp_begin[oo];
      const int32_t* cs = w.cell_start + (size_t)oo * kCellStride;
      const uint4 q0 = mp_desc[2 * (size_t)mm], q1 = mp_desc[2 * (size_t)mm + 1];
      const float2* xy = w.xy_csr + k0;
      const uint4* dsc = w.desc_csr + 2 * (size_t)k0;
      for (int ix = x0; ix <= x1; ++ix) {
        // one cell row of the rectangle is one contiguous CSR range
        const int e = cs[ix * kGridRows + y1 + 1];
        for (int p = cs[ix * kGridRows + y0] + gl; p < e; p += 2 * kGroup) {
          // two positions per lane per step: their loads are independent
          const int p2 = p + kGroup;
          const float2 a = xy[p];
          const float2 c = p2 < e ? xy[p2] : make_float2(-1e30f, -1e30f);
          const bool ia = fabsf(__fsub_rn(a.x, uu)) < rr && fabsf(__fsub_rn(a.y, vv)) < rr;
          const bool ic = fabsf(__fsub_rn(c.x, uu)) < rr && fabsf(__fsub_rn(c.y, vv)) < rr;
          uint4 a0, a1, c0, c1;
          if (ia) {
            a0 = dsc[2 * p];
            a1 = dsc[2 * p + 1];
          }
          if (ic) {
            c0 = dsc[2 * p2];
            c1 = dsc[2 * p2 + 1];
          }
          if (ia) {
            const unsigned key = (hamming32(q0, q1, a0, a1) << kPosBits) | (unsigned)p;
            const unsigned hi2 = max(key, b0);
            b0 = min(key, b0);
            b1 = min(hi2, b1);
          }
          if (ic) {
            const unsigned key = (hamming32(q0, q1, c0, c1) << kPosBits) | (unsigned)p2;
            const unsigned hi2 = max(key, b0);
            b0 = min(key, b0);
            b1 = min(hi2, b1);
          }
        }
      }
    }
    // top-2 across the group (keys are distinct)
#pragma unroll
    for (int d = 1; d < kGroup; d <<= 1) {
      const unsigned c0 = __shfl_xor_sync(0xffffffffu, b0, d);
      const unsigned c1 = __shfl_xor_sync(0xffffffffu, b1, d);
      const unsigned hi0 = max(b0, c0);
      b0 = min(b0, c0);
      b1 = min(hi0, min(b1, c1));
    }
    if (gl == 0 && mm < n_mp) {
      int match = -1;
      if (b0 != kNoKey) {
        const unsigned d0 = b0 >> kPosBits;
        const unsigned d1 = b1 != kNoKey ? (b1 >> kPosBits) : 999u;
        // MatchResKnn::FilterRatio then MatchRes::FilterThreshold (float distances)
        if ((float)d0 / (float)d1 <= ratio && !((float)d0 > (float)max_dist))
          match = w.cell_kp[k0 + (int)(b0 & (kMaxObjectKps - 1))];
      }
      mp_match[mm] = match;
      if (match >= 0) {
        atomicMax(&w.claim[k0 + match], mm - mp_begin[oo]);
        atomicAdd(&obj_count[oo], 1);
        if (mp_prev_kp) {
          const int pk = mp_prev_kp[mm];
          if (pk >= 0 && pk < kp_begin[oo + 1] - k0) w.cleared[k0 + pk] = 1;
        }
      }
    }
  }
}

__global__ void k_bind(int n_objects, int n_kp, const int32_t* __restrict__ kp_begin,
                       const int32_t* __restrict__ mp_begin, const int32_t* __restrict__ mp_id, Work w,
                       int32_t* __restrict__ kp_bind) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_kp) return;
  const int c = w.claim[k];
  if (c >= 0) {
    // the owner is the last object with kp_begin <= k (it is non-empty)
    int lo = 0, hi = n_objects - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (kp_begin[mid] <= k) lo = mid; else hi = mid - 1;
    }
    kp_bind[k] = mp_id[mp_begin[lo] + c];
  } else if (w.cleared[k]) {
    kp_bind[k] = -1;
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

size_t scratch_bytes(int n_objects, int n_kp) {
  const size_t nk = (size_t)n_kp;
  return align16((size_t)n_objects * kCellStride * 4) + align16(nk * 4) + align16(nk * 8) + align16(nk * 32) +
         align16((size_t)n_objects * 128) + align16(nk * 4) + align16(nk);
}

Work carve(void* base, int n_objects, int n_kp) {
  char* p = static_cast<char*>(base);
  const size_t nk = (size_t)n_kp;
  Work w;
  w.cell_start = reinterpret_cast<int32_t*>(p);
  p += align16((size_t)n_objects * kCellStride * 4);
  w.cell_kp = reinterpret_cast<int32_t*>(p);
  p += align16(nk * 4);
  w.xy_csr = reinterpret_cast<float2*>(p);
  p += align16(nk * 8);
  w.desc_csr = reinterpret_cast<uint4*>(p);
  p += align16(nk * 32);
  w.obj_d = reinterpret_cast<double*>(p);
  p += align16((size_t)n_objects * 128);
  w.claim = reinterpret_cast<int32_t*>(p);
  p += align16(nk * 4);
  w.cleared = reinterpret_cast<uint8_t*>(p);
  return w;
}

// every pointer of b is a device pointer
int launch(const mcba_projection_batch* b, int n_kp, int n_mp, int32_t* kp_bind, int32_t* mp_match,
           int32_t* obj_count, void* work, cudaStream_t st) {
  const Work w = carve(work, b->n_objects, n_kp);
  k_grid<<<b->n_objects, 256, 0, st>>>(b->kp_begin, b->kp_xy, reinterpret_cast<const uint4*>(b->kp_desc),
                                       b->obj_size, b->obj_Rt, w, obj_count);
  if (n_mp > 0) {
    const int warps = (n_mp + 31) / 32;
    k_project<<<(warps + 3) / 4, 128, 0, st>>>(b->n_objects, n_mp, b->mp_begin, b->obj_Rt, b->obj_K, b->obj_size,
                                              b->obj_radius, b->obj_scale, b->n_levels, b->ratio, b->max_dist,
                                              b->kp_begin, b->mp_X, reinterpret_cast<const uint4*>(b->mp_desc),
                                              b->mp_level, b->mp_prev_kp, w, mp_match, obj_count);
  }
  if (n_kp > 0)
    k_bind<<<(n_kp + 255) / 256, 256, 0, st>>>(b->n_objects, n_kp, b->kp_begin, b->mp_begin, b->mp_id, w, kp_bind);
  return cudaGetLastError() == cudaSuccess ? MCBA_OK : MCBA_ERR_CUDA;
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

}  // namespace

extern "C" int mcba_project_match_device(const mcba_projection_batch* b, int32_t n_kp, int32_t n_mp,
                                         int32_t* kp_bind, int32_t* mp_match, int32_t* obj_count, void* stream) {
  if (!b || b->n_objects < 0 || n_kp < 0 || n_mp < 0 || b->n_levels <= 0) return MCBA_ERR_INVALID;
  if (b->n_objects == 0) return MCBA_OK;
  if (!b->obj_Rt || !b->obj_K || !b->obj_size || !b->obj_radius || !b->obj_scale || !b->kp_begin ||
      !b->mp_begin || !obj_count)
    return MCBA_ERR_INVALID;
  if (n_kp > 0 && (!b->kp_xy || !b->kp_desc || !kp_bind || !aligned16(b->kp_desc) ||
                   (reinterpret_cast<uintptr_t>(b->kp_xy) & 7u)))
    return MCBA_ERR_INVALID;
  if (n_mp > 0 && (!b->mp_X || !b->mp_desc || !b->mp_level || !b->mp_id || !mp_match || !aligned16(b->mp_desc)))
    return MCBA_ERR_INVALID;
  int dev = 0;
  cudaGetDevice(&dev);
  void* work = nullptr;
  if (scratch(dev, scratch_bytes(b->n_objects, n_kp), &work) != cudaSuccess) return MCBA_ERR_NOMEM;
  return launch(b, n_kp, n_mp, kp_bind, mp_match, obj_count, work, static_cast<cudaStream_t>(stream));
}

extern "C" int mcba_project_match(int32_t device, const mcba_projection_batch* b, int32_t* kp_bind,
                                  int32_t* mp_match, int32_t* obj_count, double* ms_device) {
  if (!b || b->n_objects < 0 || b->n_levels <= 0) return MCBA_ERR_INVALID;
  const int O = b->n_objects;
  if (ms_device) *ms_device = 0.0;
  if (O == 0) return MCBA_OK;
  if (!b->obj_Rt || !b->obj_K || !b->obj_size || !b->obj_radius || !b->obj_scale || !b->kp_begin ||
      !b->mp_begin || !obj_count)
    return MCBA_ERR_INVALID;
  // host-side validation: ranges, sizes, levels, finite inputs
  if (b->kp_begin[0] != 0 || b->mp_begin[0] != 0) return MCBA_ERR_INVALID;
  for (int o = 0; o < O; ++o) {
    if (b->kp_begin[o + 1] < b->kp_begin[o] || b->mp_begin[o + 1] < b->mp_begin[o]) return MCBA_ERR_INVALID;
    if (b->kp_begin[o + 1] - b->kp_begin[o] >= kMaxObjectKps) return MCBA_ERR_TOO_LARGE;
    if (b->obj_size[2 * o] <= 0 || b->obj_size[2 * o + 1] <= 0) return MCBA_ERR_INVALID;
    for (int k = 0; k < 12; ++k)
      if (!std::isfinite(b->obj_Rt[12 * (size_t)o + k])) return MCBA_ERR_NONFINITE;
    for (int k = 0; k < 4; ++k)
      if (!std::isfinite(b->obj_K[4 * (size_t)o + k])) return MCBA_ERR_NONFINITE;
    if (!std::isfinite(b->obj_radius[o])) return MCBA_ERR_NONFINITE;
  }
  const int n_kp = b->kp_begin[O], n_mp = b->mp_begin[O];
  if (n_kp > 0 && (!b->kp_xy || !b->kp_desc || !kp_bind)) return MCBA_ERR_INVALID;
  if (n_mp > 0 && (!b->mp_X || !b->mp_desc || !b->mp_level || !b->mp_id || !mp_match)) return MCBA_ERR_INVALID;
  for (int k = 0; k < 2 * n_kp; ++k)
    if (!std::isfinite(b->kp_xy[k])) return MCBA_ERR_NONFINITE;
  for (int m = 0; m < n_mp; ++m) {
    if (b->mp_level[m] < 0 || b->mp_level[m] >= b->n_levels) return MCBA_ERR_INVALID;
    if (!std::isfinite(b->mp_X[3 * (size_t)m]) || !std::isfinite(b->mp_X[3 * (size_t)m + 1]) ||
        !std::isfinite(b->mp_X[3 * (size_t)m + 2]))
      return MCBA_ERR_NONFINITE;
  }
  if (b->mp_prev_kp)
    for (int o = 0; o < O; ++o)
      for (int m = b->mp_begin[o]; m < b->mp_begin[o + 1]; ++m)
        if (b->mp_prev_kp[m] < -1 || b->mp_prev_kp[m] >= b->kp_begin[o + 1] - b->kp_begin[o]) return MCBA_ERR_INVALID;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return MCBA_ERR_NO_DEVICE;
  if (device < 0 || device >= n || cudaSetDevice(device) != cudaSuccess) return MCBA_ERR_INVALID;

  // one device allocation holds every input, output and the scratch
  const size_t L = (size_t)b->n_levels;
  struct Part {
    const void* src;
    size_t bytes;
    size_t off;
  };
  std::vector<Part> parts = {
      {b->obj_Rt, 48 * (size_t)O, 0},          {b->obj_K, 16 * (size_t)O, 0},
      {b->obj_size, 8 * (size_t)O, 0},         {b->obj_radius, 4 * (size_t)O, 0},
      {b->obj_scale, 4 * L * O, 0},            {b->kp_begin, 4 * (size_t)(O + 1), 0},
      {b->kp_xy, 8 * (size_t)n_kp, 0},         {b->kp_desc, 32 * (size_t)n_kp, 0},
      {b->mp_begin, 4 * (size_t)(O + 1), 0},   {b->mp_X, 12 * (size_t)n_mp, 0},
      {b->mp_desc, 32 * (size_t)n_mp, 0},      {b->mp_level, 4 * (size_t)n_mp, 0},
      {b->mp_id, 4 * (size_t)n_mp, 0},         {b->mp_prev_kp, b->mp_prev_kp ? 4 * (size_t)n_mp : 0, 0},
      {kp_bind, 4 * (size_t)n_kp, 0},          {nullptr, 4 * (size_t)n_mp, 0},
      {nullptr, 4 * (size_t)O, 0},             {nullptr, scratch_bytes(O, n_kp), 0}};
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
    mcba_projection_batch d = *b;
    d.obj_Rt = static_cast<const float*>(at(0));
    d.obj_K = static_cast<const float*>(at(1));
    d.obj_size = static_cast<const int32_t*>(at(2));
    d.obj_radius = static_cast<const float*>(at(3));
    d.obj_scale = static_cast<const float*>(at(4));
    d.kp_begin = static_cast<const int32_t*>(at(5));
    d.kp_xy = static_cast<const float*>(at(6));
    d.kp_desc = static_cast<const uint8_t*>(at(7));
    d.mp_begin = static_cast<const int32_t*>(at(8));
    d.mp_X = static_cast<const float*>(at(9));
    d.mp_desc = static_cast<const uint8_t*>(at(10));
    d.mp_level = static_cast<const int32_t*>(at(11));
    d.mp_id = static_cast<const int32_t*>(at(12));
    d.mp_prev_kp = b->mp_prev_kp ? static_cast<const int32_t*>(at(13)) : nullptr;
    int32_t* d_bind = static_cast<int32_t*>(at(14));
    int32_t* d_match = static_cast<int32_t*>(at(15));
    int32_t* d_count = static_cast<int32_t*>(at(16));
    cudaEventRecord(e0, st);
    r = launch(&d, n_kp, n_mp, d_bind, d_match, d_count, at(17), st);
    cudaEventRecord(e1, st);
    if (r) break;
    r = MCBA_ERR_CUDA;
    if (n_kp && cudaMemcpyAsync(kp_bind, d_bind, 4 * (size_t)n_kp, cudaMemcpyDeviceToHost, st) != cudaSuccess) break;
    if (n_mp && cudaMemcpyAsync(mp_match, d_match, 4 * (size_t)n_mp, cudaMemcpyDeviceToHost, st) != cudaSuccess)
      break;
    if (cudaMemcpyAsync(obj_count, d_count, 4 * (size_t)O, cudaMemcpyDeviceToHost, st) != cudaSuccess) break;
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
