// mcba_window.cu -- the local-BA window of a new keyframe, chosen and
// assembled on the GPU from flat map tables.
//
// What Map::AddKeyFrame does before its local bundle adjustment
// (src/Map.cpp:140-145), with the hash-set walks replaced by flag arrays,
// scans and segmented counts:
//   GrabLocalMap_Mappoint(frame, hop)   keyframes bound to the frame's LEFT
//                                       map points, widened hop-1 times over
//                                       the essential graph, the frame
//                                       itself removed (src/Map.cpp:730-756)
//   GrabAnchorKeyFrames(kfs)            the essential-graph neighbours of the
//                                       smallest-id keyframe with a smaller
//                                       id still (src/Map.cpp:775-796)
//   ThisMapPointBeFix(mp, kfs, fix)     per map point, the bound keyframes
//                                       counted in the window and among the
//                                       anchors; fixed iff
//                                       (n_free + 1) / (n_fix + 1) <= 1.5
//                                       (src/PoseEstimation.cpp:153-163)
//   BoundleAdjustment's insertion loop  anchors then window keyframes, each
//                                       with its LEFT then WIDE observations;
//                                       a map point takes its vertex id at
//                                       its first edge
//                                       (include/PoseEstimation.hpp:36-97,
//                                       src/BAoptimizer.cpp:22-108)
// A set of keyframes is walked in ascending map index (the reference's
// unordered_set order is unspecified) and the observations of one object in
// table order.
//
// Kernels, one stream, one host synchronisation at the end:
//   k_win_seed     one thread per LEFT observation of the frame: marks the
//                  keyframes bound to its map point
//   k_win_hop      one breadth-first round over the essential graph
//   k_win_plan     one CTA: frame removed, smallest id, anchors, roles,
//                  pose numbering, per-keyframe segments and edge offsets
//   k_win_emit     one CTA per segment: LEFT then WIDE observations ranked
//                  by block scans into the edge order; first edge of each
//                  map point by atomicMin
//   k_scan_*       exclusive scan of the first-edge flags -> point ids
//   k_win_points   per new point: map index, ThisMapPointBeFix
//   k_win_edges    per edge: the bulk-loader arrays of the problem
// Every table index is checked against its table; a bad index or range sets
// an error word and the access is skipped.

#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "mcba.h"
#include "mcba_internal.h"
#include "mcba_window.h"

namespace mcba {
namespace {

constexpr int kWinThreads = 256;
constexpr int kPlanThreads = 1024;
constexpr int kScanBlock = 1024;  // elements per scan block (256 threads x 4)
constexpr float kMinDisparity = 1.f;  // MIN_DISPARITY, include/PoseEstimation.hpp:14

enum : int { kErrIndex = 1, kErrRange = 2 };

// Device copy of the map tables.
struct MapDev {
  int K, P, O, B, A, L;
  const long long* kf_id;
  const int* obs_begin;
  const int* obs_point;
  const uint8_t* obs_object;
  const float* obs_uv;
  const float* obs_ur;
  const uint8_t* obs_octave;
  const int* mp_kf_begin;
  const int* mp_kf;
  const int* ess_begin;
  const int* ess_adj;
  const float* inv_s2_left;
  const float* inv_s2_wide;
};

// Window state and outputs.
struct WinDev {
  uint8_t* inset;     // [K] in GrabLocalMap_Mappoint's set
  uint8_t* front;     // [K] current breadth-first frontier
  uint8_t* next;      // [K]
  uint8_t* role;      // [K] bit 0 optimised, bit 1 anchor
  int* pose_of_kf;    // [K]
  int* seg_kf;        // [2K] keyframe of each segment
  int* seg_off;       // [2K + 1] first edge of each segment
  int* pose_kf;       // [K] map keyframe of each problem pose
  uint8_t* pose_fixed;// [K]
  int* counts;        // [8]: nseg, n_edges, n_poses, n_local, n_anchor, n_points, n_fixed_points, error
  int* first_edge;    // [P] smallest edge index of each map point
  int* mp_pid;        // [P] problem point id of each map point in the window
  int* edge_obs;      // [O] table row of each edge
  int* edge_seg;      // [O]
  int* flag;          // [O + 1] first-edge flags, then their exclusive scan
  int* scan_sums;     // scan block sums
  int* point_mp;      // [P]
  uint8_t* point_fixed;  // [P]
  // problem edges
  uint8_t* e_type;
  int* e_pose;
  int* e_point;
  int* e_cam;
  float* e_obs;       // [O][3]
  float* e_info;
  float* e_delta;
};

enum { kCntSeg = 0, kCntEdges, kCntPoses, kCntLocal, kCntAnchor, kCntPoints, kCntFixedPts, kCntError, kCnt };

__device__ __forceinline__ void set_error(int* counts, int code) { atomicOr(&counts[kCntError], code); }

// A CSR range [begin[i], begin[i+1]) checked against the table length.
__device__ __forceinline__ bool csr_range(const int* begin, int i, int total, int* counts, int& b0, int& b1) {
  b0 = begin[i];
  b1 = begin[i + 1];
  if (b0 < 0 || b1 < b0 || b1 > total) {
    set_error(counts, kErrRange);
    return false;
  }
  return true;
}

// GrabLocalMap_Mappoint, first part: every keyframe bound to a map point of
// the frame's LEFT object joins the set (and the first frontier).
__global__ void __launch_bounds__(kWinThreads) k_win_seed(MapDev m, WinDev w, int cur) {
  int o0, o1;
  if (!csr_range(m.obs_begin, cur, m.O, w.counts, o0, o1)) return;
  const int o = o0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= o1 || m.obs_object[o] != 0) return;
  const int mp = m.obs_point[o];
  if (mp < 0 || mp >= m.P) {
    set_error(w.counts, kErrIndex);
    return;
  }
  int b0, b1;
  if (!csr_range(m.mp_kf_begin, mp, m.B, w.counts, b0, b1)) return;
  for (int b = b0; b < b1; ++b) {
    const int kf = m.mp_kf[b];
    if (kf < 0 || kf >= m.K) {
      set_error(w.counts, kErrIndex);
      continue;
    }
    w.inset[kf] = 1;
    w.front[kf] = 1;
  }
}

// One breadth-first round (src/Map.cpp:741-751): neighbours of the frontier
// not yet in the set join it and form the next frontier.  Concurrent joins
// of one keyframe store the same values, so the result is the sequential
// round's.
__global__ void __launch_bounds__(kWinThreads) k_win_hop(MapDev m, WinDev w) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m.K || !w.front[k]) return;
  int a0, a1;
  if (!csr_range(m.ess_begin, k, m.A, w.counts, a0, a1)) return;
  for (int a = a0; a < a1; ++a) {
    const int to = m.ess_adj[a];
    if (to < 0 || to >= m.K) {
      set_error(w.counts, kErrIndex);
      continue;
    }
    if (!w.inset[to]) {
      w.inset[to] = 1;
      w.next[to] = 1;
    }
  }
}

// Inclusive block scan of one int per thread (kPlanThreads threads).
__device__ __forceinline__ int block_incl_scan(int v, int* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  if (lane == 31) sh[wid] = v;
  __syncthreads();
  if (wid == 0) {
    int s = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += t;
    }
    sh[lane] = s;
  }
  __syncthreads();
  const int add = wid ? sh[wid - 1] : 0;
  __syncthreads();
  return v + add;
}

// One CTA: the frame leaves the set (src/Map.cpp:754), the smallest-id
// keyframe of the set and its older essential-graph neighbours become the
// anchors (src/Map.cpp:775-796), the frame joins the window
// (src/Map.cpp:144); then the insertion loop's order
// (include/PoseEstimation.hpp:40,70): one segment per anchor, then one per
// window keyframe, ascending map index; a keyframe takes its pose id at its
// first segment (BAoptimizer::addKeyFrame ignores a second add).
__global__ void __launch_bounds__(kPlanThreads) k_win_plan(MapDev m, WinDev w, int cur) {
  __shared__ int sh[32];
  __shared__ unsigned long long best;
  __shared__ int kmin, carry, carry2;
  const int K = m.K;
  if (threadIdx.x == 0) {
    w.inset[cur] = 0;
    best = ULLONG_MAX;
  }
  __syncthreads();
  // smallest Frame::id in the set (ids are unique; id then index as the key)
  unsigned long long mine = ULLONG_MAX;
  for (int k = threadIdx.x; k < K; k += blockDim.x)
    if (w.inset[k]) {
      const unsigned long long key = ((unsigned long long)m.kf_id[k] << 24) | (unsigned long long)k;
      mine = key < mine ? key : mine;
    }
  atomicMin(&best, mine);
  __syncthreads();
  if (threadIdx.x == 0) kmin = (best == ULLONG_MAX) ? -1 : (int)(best & 0xffffffull);
  __syncthreads();
  for (int k = threadIdx.x; k < K; k += blockDim.x) w.role[k] = w.inset[k] ? 1 : 0;
  __syncthreads();
  if (kmin >= 0) {
    int a0, a1;
    if (csr_range(m.ess_begin, kmin, m.A, w.counts, a0, a1))
      for (int a = a0 + threadIdx.x; a < a1; a += blockDim.x) {
        const int to = m.ess_adj[a];
        if (to < 0 || to >= K) {
          set_error(w.counts, kErrIndex);
          continue;
        }
        if (to != kmin && m.kf_id[to] < m.kf_id[kmin]) w.role[to] |= 2;  // same value from every writer
      }
  }
  __syncthreads();
  if (threadIdx.x == 0) w.role[cur] |= 1;
  __syncthreads();
  // anchor segments (ascending index): pose ids 0 .. n_anchor-1, fixed
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < K; base += blockDim.x) {
    const int k = base + threadIdx.x;
    const int f = (k < K && (w.role[k] & 2)) ? 1 : 0;
    const int inc = block_incl_scan(f, sh);
    if (f) {
      const int s = carry + inc - 1;
      w.seg_kf[s] = k;
      w.pose_of_kf[k] = s;
      w.pose_kf[s] = k;
      w.pose_fixed[s] = 1;
    }
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry += inc;
    __syncthreads();
  }
  const int n_anchor = carry;
  // window segments (ascending index); keyframes not already anchors take
  // the next pose ids, fixed only when Frame::id == 0 (src/BAoptimizer.cpp:30)
  __syncthreads();
  if (threadIdx.x == 0) {
    carry = 0;
    carry2 = 0;
  }
  __syncthreads();
  for (int base = 0; base < K; base += blockDim.x) {
    const int k = base + threadIdx.x;
    const int f = (k < K && (w.role[k] & 1)) ? 1 : 0;
    const int g = (f && !(w.role[k] & 2)) ? 1 : 0;
    const int inc = block_incl_scan(f, sh);
    const int inc2 = block_incl_scan(g, sh);
    if (f) w.seg_kf[n_anchor + carry + inc - 1] = k;
    if (g) {
      const int pid = n_anchor + carry2 + inc2 - 1;
      w.pose_of_kf[k] = pid;
      w.pose_kf[pid] = k;
      w.pose_fixed[pid] = m.kf_id[k] == 0 ? 1 : 0;
    }
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) {
      carry += inc;
      carry2 += inc2;
    }
    __syncthreads();
  }
  const int n_local = carry, nseg = n_anchor + carry;
  // edge offsets of the segments
  __syncthreads();
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nseg; base += blockDim.x) {
    const int s = base + threadIdx.x;
    int c = 0;
    if (s < nseg) {
      int o0, o1;
      if (csr_range(m.obs_begin, w.seg_kf[s], m.O, w.counts, o0, o1)) c = o1 - o0;
    }
    const int inc = block_incl_scan(c, sh);
    if (s < nseg) w.seg_off[s] = carry + inc - c;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry += inc;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    w.seg_off[nseg] = carry;
    w.counts[kCntSeg] = nseg;
    w.counts[kCntEdges] = carry;
    w.counts[kCntPoses] = n_anchor + carry2;
    w.counts[kCntLocal] = n_local;
    w.counts[kCntAnchor] = n_anchor;
  }
}

// One CTA per segment: the keyframe's LEFT observations, then its WIDE
// observations, each in table order (include/PoseEstimation.hpp:42,60), get
// consecutive edge indices from block scans.  The first edge of a map point
// gives it its vertex id (BAoptimizer::addMapppint ignores later adds).
__global__ void __launch_bounds__(kWinThreads) k_win_emit(MapDev m, WinDev w) {
  __shared__ int sh[32];
  __shared__ int carry;
  const int s = blockIdx.x;
  if (s >= w.counts[kCntSeg]) return;
  const int kf = w.seg_kf[s];
  int o0, o1;
  if (!csr_range(m.obs_begin, kf, m.O, w.counts, o0, o1)) return;
  if (threadIdx.x == 0) carry = w.seg_off[s];
  __syncthreads();
  for (int obj = 0; obj < 2; ++obj)
    for (int base = o0; base < o1; base += blockDim.x) {
      const int o = base + threadIdx.x;
      int f = 0;
      if (o < o1) {
        const int ob = m.obs_object[o];
        f = (obj == 0) ? (ob == 0) : (ob != 0);
        if (obj == 1 && ob > 1) set_error(w.counts, kErrIndex);
      }
      // inclusive scan over the CTA (blockDim.x = kWinThreads)
      const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
      int v = f;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d) v += t;
      }
      if (lane == 31) sh[wid] = v;
      __syncthreads();
      if (wid == 0) {
        int t = (lane < kWinThreads / 32) ? sh[lane] : 0;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          const int u = __shfl_up_sync(0xffffffffu, t, d);
          if (lane >= d) t += u;
        }
        sh[lane] = t;
      }
      __syncthreads();
      const int inc = v + (wid ? sh[wid - 1] : 0);
      if (f) {
        const int e = carry + inc - 1;
        w.edge_obs[e] = o;
        w.edge_seg[e] = s;
        const int mp = m.obs_point[o];
        if (mp < 0 || mp >= m.P)
          set_error(w.counts, kErrIndex);
        else
          atomicMin(&w.first_edge[mp], e);
      }
      __syncthreads();
      if (threadIdx.x == blockDim.x - 1) carry += inc;
      __syncthreads();
    }
}

// flag[e] = 1 where edge e is its map point's first edge.
__global__ void k_win_first(MapDev m, WinDev w) {
  const int E = w.counts[kCntEdges];
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e > E) return;
  int f = 0;
  if (e < E) {
    const int mp = m.obs_point[w.edge_obs[e]];
    f = (mp >= 0 && mp < m.P && w.first_edge[mp] == e) ? 1 : 0;
  }
  w.flag[e] = f;
}

// Exclusive scan of flag[0..E] in place (E read on the device), 1024
// elements per block; block totals to sums.
__global__ void __launch_bounds__(256) k_scan_block(int* a, const int* n_dev, int* sums) {
  __shared__ int sh[8];
  const int n = *n_dev + 1;
  const int base = blockIdx.x * kScanBlock + threadIdx.x * 4;
  if (blockIdx.x * kScanBlock >= n) return;
  int v[4], s = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    v[i] = (base + i < n) ? a[base + i] : 0;
    s += v[i];
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int inc = s;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, inc, d);
    if (lane >= d) inc += t;
  }
  if (lane == 31) sh[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    int t = lane < 8 ? sh[lane] : 0;
#pragma unroll
    for (int d = 1; d < 8; d <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, t, d);
      if (lane >= d) t += u;
    }
    if (lane < 8) sh[lane] = t;
  }
  __syncthreads();
  int run = inc - s + (wid ? sh[wid - 1] : 0);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    if (base + i < n) a[base + i] = run;
    run += v[i];
  }
  if (threadIdx.x == 255) sums[blockIdx.x] = run;
}

// Exclusive scan of the block sums (one CTA, any count).
__global__ void __launch_bounds__(1024) k_scan_sums(int* sums, const int* n_dev) {
  __shared__ int sh[32];
  __shared__ int carry;
  const int nb = (*n_dev + 1 + kScanBlock - 1) / kScanBlock;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nb; base += blockDim.x) {
    const int i = base + threadIdx.x;
    const int v = i < nb ? sums[i] : 0;
    const int inc = block_incl_scan(v, sh);
    if (i < nb) sums[i] = carry + inc - v;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry += inc;
    __syncthreads();
  }
}

__global__ void k_scan_add(int* a, const int* n_dev, const int* sums) {
  const int n = *n_dev + 1;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] += sums[i / kScanBlock];  // sums[0] is 0
}

// Each map point at its first edge: its problem id, position and
// ThisMapPointBeFix over its bound keyframes (src/PoseEstimation.cpp:153-163):
// a keyframe in the window counts as free, else an anchor as fixed; fixed iff
// (n_free + 1) / (n_fix + 1) <= 1.5, i.e. 2 (n_free + 1) <= 3 (n_fix + 1) --
// the quotient of two small integers rounds to exactly 1.5 only when it is 1.5.
__global__ void k_win_points(MapDev m, WinDev w) {
  const int E = w.counts[kCntEdges];
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  const int pid = w.flag[e];
  if (w.flag[e + 1] == pid) return;  // not a first edge
  const int mp = m.obs_point[w.edge_obs[e]];
  w.mp_pid[mp] = pid;
  w.point_mp[pid] = mp;
  int b0, b1;
  int n_free = 0, n_fix = 0;
  if (csr_range(m.mp_kf_begin, mp, m.B, w.counts, b0, b1))
    for (int b = b0; b < b1; ++b) {
      const int kf = m.mp_kf[b];
      if (kf < 0 || kf >= m.K) {
        set_error(w.counts, kErrIndex);
        continue;
      }
      const int r = w.role[kf];
      if (r & 1)
        ++n_free;
      else if (r & 2)
        ++n_fix;
    }
  const bool fixed = 2 * (n_free + 1) <= 3 * (n_fix + 1);
  w.point_fixed[pid] = fixed ? 1 : 0;
  if (fixed) atomicAdd(&w.counts[kCntFixedPts], 1);
}

// The problem's edges (BAoptimizer::addEdge / addEdgeStereo / addEdgeToBody,
// src/BAoptimizer.cpp:45-108): LEFT with u_right != -1 and >= MIN_DISPARITY
// is a stereo edge (include/PoseEstimation.hpp:52), other LEFT observations
// mono edges of camera 0 (T_cam_body = I), WIDE observations mono edges of
// camera 1 (kf->Twl); information = mvInvLevelSigma2[octave] of the object's
// extractor; Huber thresholds sqrt(5.99) for LEFT mono, sqrt(7.815) otherwise.
__global__ void k_win_edges(MapDev m, WinDev w, float th2d, float th3d) {
  const int E = w.counts[kCntEdges];
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e == 0) w.counts[kCntPoints] = w.flag[E];
  if (e >= E) return;
  const int o = w.edge_obs[e];
  const int kf = w.seg_kf[w.edge_seg[e]];
  const int mp = m.obs_point[o];
  if (mp < 0 || mp >= m.P) return;  // flagged by k_win_emit
  const bool left = m.obs_object[o] == 0;
  const float ur = m.obs_ur[o];
  const bool stereo = left && ur != -1.f && ur >= kMinDisparity;
  const int lv = m.obs_octave[o];
  float info = 0.f;
  if (lv >= m.L)
    set_error(w.counts, kErrIndex);
  else
    info = left ? m.inv_s2_left[lv] : m.inv_s2_wide[lv];
  w.e_type[e] = stereo ? MCBA_EDGE_STEREO : MCBA_EDGE_MONO;
  w.e_pose[e] = w.pose_of_kf[kf];
  w.e_point[e] = w.mp_pid[mp];
  w.e_cam[e] = left ? 0 : 1;
  w.e_obs[3 * (size_t)e] = m.obs_uv[2 * (size_t)o];
  w.e_obs[3 * (size_t)e + 1] = m.obs_uv[2 * (size_t)o + 1];
  w.e_obs[3 * (size_t)e + 2] = stereo ? ur : 0.f;
  w.e_info[e] = info;
  w.e_delta[e] = (left && !stereo) ? th2d : th3d;
}

#define WCK(call)                                                                  \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess) {                                                       \
      if (err) *err = std::string(#call) + ": " + cudaGetErrorString(e_);          \
      return MCBA_ERR_CUDA;                                                        \
    }                                                                              \
  } while (0)

// Per-device workspace (buffers grow, never shrink).
struct WinWorkspace {
  cudaStream_t stream = nullptr;
  DBuf<char> map;   // the uploaded tables, one allocation
  DBuf<char> win;   // window state and outputs
  char* pinned = nullptr;  // staging for the read-back
  size_t pinned_cap = 0;
};
std::mutex g_win_mutex;
std::vector<WinWorkspace*> g_win_ws;

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

template <typename T>
T* carve(char*& p, size_t n) {
  T* r = reinterpret_cast<T*>(p);
  p += align256(n * sizeof(T));
  return r;
}

}  // namespace

int window_assemble(int device, const mcba_map_desc* d, int32_t cur, int32_t hop, WindowHost& out,
                    std::string* err) {
  const int K = d->n_keyframes, P = d->n_points;
  const int O = d->obs_begin[K], B = d->mp_kf_begin[P], A = d->ess_begin[K], L = d->n_levels;
  std::lock_guard<std::mutex> lock(g_win_mutex);
  WCK(cudaSetDevice(device));
  if ((int)g_win_ws.size() <= device) g_win_ws.resize(device + 1, nullptr);
  if (!g_win_ws[device]) {
    g_win_ws[device] = new WinWorkspace();
    WCK(cudaStreamCreateWithFlags(&g_win_ws[device]->stream, cudaStreamNonBlocking));
  }
  WinWorkspace& ws = *g_win_ws[device];
  cudaStream_t st = ws.stream;

  // tables: one allocation, one copy per array
  struct Piece {
    const void* src;
    size_t bytes;
  };
  const Piece pieces[] = {
      {d->kf_id, sizeof(int64_t) * K},          {d->obs_begin, sizeof(int32_t) * (K + 1)},
      {d->obs_point, sizeof(int32_t) * O},      {d->obs_object, (size_t)O},
      {d->obs_uv, sizeof(float) * 2 * O},       {d->obs_ur, sizeof(float) * O},
      {d->obs_octave, (size_t)O},               {nullptr, 0},
      {d->mp_kf_begin, sizeof(int32_t) * (P + 1)}, {d->mp_kf, sizeof(int32_t) * B},
      {d->ess_begin, sizeof(int32_t) * (K + 1)}, {d->ess_adj, sizeof(int32_t) * A},
      {d->inv_sigma2_left, sizeof(float) * L},  {d->inv_sigma2_wide, sizeof(float) * L}};
  constexpr int NP = sizeof(pieces) / sizeof(pieces[0]);
  size_t total = 0;
  for (const Piece& pc : pieces) total += align256(pc.bytes);
  WCK(ws.map.ensure(total));
  const void* dev[NP];
  {
    char* p = ws.map.p;
    for (int i = 0; i < NP; ++i) {
      dev[i] = p;
      if (pieces[i].bytes) WCK(cudaMemcpyAsync(p, pieces[i].src, pieces[i].bytes, cudaMemcpyHostToDevice, st));
      p += align256(pieces[i].bytes);
    }
  }
  MapDev m;
  m.K = K;
  m.P = P;
  m.O = O;
  m.B = B;
  m.A = A;
  m.L = L;
  m.kf_id = static_cast<const long long*>(dev[0]);
  m.obs_begin = static_cast<const int*>(dev[1]);
  m.obs_point = static_cast<const int*>(dev[2]);
  m.obs_object = static_cast<const uint8_t*>(dev[3]);
  m.obs_uv = static_cast<const float*>(dev[4]);
  m.obs_ur = static_cast<const float*>(dev[5]);
  m.obs_octave = static_cast<const uint8_t*>(dev[6]);
  m.mp_kf_begin = static_cast<const int*>(dev[8]);
  m.mp_kf = static_cast<const int*>(dev[9]);
  m.ess_begin = static_cast<const int*>(dev[10]);
  m.ess_adj = static_cast<const int*>(dev[11]);
  m.inv_s2_left = static_cast<const float*>(dev[12]);
  m.inv_s2_wide = static_cast<const float*>(dev[13]);

  // window workspace: every edge is one observation of the table, so O
  // bounds the edge count (a keyframe that is both anchor and window member
  // contributes twice: 2 O)
  const size_t Emax = 2 * (size_t)O;
  const int nsb = (int)((Emax + 1 + kScanBlock - 1) / kScanBlock) + 1;
  const size_t need = align256(K) * 4 + align256(sizeof(int) * K) * 2 + align256(sizeof(int) * 2 * (size_t)K) +
                      align256(sizeof(int) * (2 * (size_t)K + 1)) + align256(K) + align256(sizeof(int) * kCnt) +
                      align256(sizeof(int) * (size_t)P) * 3 + align256(P) +
                      align256(sizeof(int) * Emax) * 2 + align256(sizeof(int) * (Emax + 1)) +
                      align256(sizeof(int) * nsb) + align256(Emax) + align256(sizeof(int) * Emax) * 3 +
                      align256(sizeof(float) * 3 * Emax) + align256(sizeof(float) * Emax) * 2;
  WCK(ws.win.ensure(need));
  WinDev w;
  {
    char* p = ws.win.p;
    w.inset = carve<uint8_t>(p, K);
    w.front = carve<uint8_t>(p, K);
    w.next = carve<uint8_t>(p, K);
    w.role = carve<uint8_t>(p, K);
    w.pose_of_kf = carve<int>(p, K);
    w.pose_kf = carve<int>(p, K);
    w.seg_kf = carve<int>(p, 2 * (size_t)K);
    w.seg_off = carve<int>(p, 2 * (size_t)K + 1);
    w.pose_fixed = carve<uint8_t>(p, K);
    w.counts = carve<int>(p, kCnt);
    w.first_edge = carve<int>(p, P);
    w.mp_pid = carve<int>(p, P);
    w.point_mp = carve<int>(p, P);
    w.point_fixed = carve<uint8_t>(p, P);
    w.edge_obs = carve<int>(p, Emax);
    w.edge_seg = carve<int>(p, Emax);
    w.flag = carve<int>(p, Emax + 1);
    w.scan_sums = carve<int>(p, nsb);
    w.e_type = carve<uint8_t>(p, Emax);
    w.e_pose = carve<int>(p, Emax);
    w.e_point = carve<int>(p, Emax);
    w.e_cam = carve<int>(p, Emax);
    w.e_obs = carve<float>(p, 3 * Emax);
    w.e_info = carve<float>(p, Emax);
    w.e_delta = carve<float>(p, Emax);
  }
  WCK(cudaMemsetAsync(w.inset, 0, (size_t)K, st));
  WCK(cudaMemsetAsync(w.front, 0, (size_t)K, st));
  WCK(cudaMemsetAsync(w.next, 0, (size_t)K, st));
  WCK(cudaMemsetAsync(w.counts, 0, sizeof(int) * kCnt, st));
  WCK(cudaMemsetAsync(w.first_edge, 0x7f, sizeof(int) * (size_t)P, st));

  const int n_cur = d->obs_begin[cur + 1] - d->obs_begin[cur];
  if (n_cur > 0) k_win_seed<<<(n_cur + kWinThreads - 1) / kWinThreads, kWinThreads, 0, st>>>(m, w, cur);
  for (int r = 1; r < hop; ++r) {
    k_win_hop<<<(K + kWinThreads - 1) / kWinThreads, kWinThreads, 0, st>>>(m, w);
    std::swap(w.front, w.next);
    WCK(cudaMemsetAsync(w.next, 0, (size_t)K, st));
  }
  k_win_plan<<<1, kPlanThreads, 0, st>>>(m, w, cur);
  k_win_emit<<<2 * K, kWinThreads, 0, st>>>(m, w);
  const int eb = (int)((Emax + 1 + 255) / 256);
  k_win_first<<<eb, 256, 0, st>>>(m, w);
  const int* n_dev = &w.counts[kCntEdges];
  k_scan_block<<<nsb, 256, 0, st>>>(w.flag, n_dev, w.scan_sums);
  k_scan_sums<<<1, 1024, 0, st>>>(w.scan_sums, n_dev);
  k_scan_add<<<eb, 256, 0, st>>>(w.flag, n_dev, w.scan_sums);
  k_win_points<<<eb, 256, 0, st>>>(m, w);
  const float th2d = (float)std::sqrt(5.99), th3d = (float)std::sqrt(7.815);  // BAoptimizer.hpp:62-63
  k_win_edges<<<eb, 256, 0, st>>>(m, w, th2d, th3d);
  WCK(cudaGetLastError());

  // read-back: sizes first, then every output in one pinned block
  int cnt[kCnt];
  WCK(cudaMemcpyAsync(cnt, w.counts, sizeof(cnt), cudaMemcpyDeviceToHost, st));
  WCK(cudaStreamSynchronize(st));
  if (cnt[kCntError]) {
    if (err) *err = (cnt[kCntError] & kErrRange) ? "map table: bad CSR range" : "map table: index out of range";
    return MCBA_ERR_INVALID;
  }
  const int E = cnt[kCntEdges], NPo = cnt[kCntPoses], NPt = cnt[kCntPoints];
  out.n_local = cnt[kCntLocal];
  out.n_anchor = cnt[kCntAnchor];
  out.n_fixed_points = cnt[kCntFixedPts];
  out.kf_role.resize(K);
  out.pose_kf.resize(NPo);
  out.pose_fixed.resize(NPo);
  out.point_mp.resize(NPt);
  out.point_fixed.resize(NPt);
  out.e_type.resize(E);
  out.e_pose.resize(E);
  out.e_point.resize(E);
  out.e_cam.resize(E);
  out.e_obs.resize(3 * (size_t)E);
  out.e_info.resize(E);
  out.e_delta.resize(E);
  struct Back {
    void* dst;
    const void* src;
    size_t bytes;
  };
  const Back back[] = {{out.kf_role.data(), w.role, (size_t)K},
                       {out.pose_kf.data(), w.pose_kf, sizeof(int) * NPo},
                       {out.pose_fixed.data(), w.pose_fixed, (size_t)NPo},
                       {out.point_mp.data(), w.point_mp, sizeof(int) * NPt},
                       {out.point_fixed.data(), w.point_fixed, (size_t)NPt},
                       {out.e_type.data(), w.e_type, (size_t)E},
                       {out.e_pose.data(), w.e_pose, sizeof(int) * E},
                       {out.e_point.data(), w.e_point, sizeof(int) * E},
                       {out.e_cam.data(), w.e_cam, sizeof(int) * E},
                       {out.e_obs.data(), w.e_obs, sizeof(float) * 3 * E},
                       {out.e_info.data(), w.e_info, sizeof(float) * E},
                       {out.e_delta.data(), w.e_delta, sizeof(float) * E}};
  size_t tot = 0;
  for (const Back& b : back) tot += align256(b.bytes);
  if (ws.pinned_cap < tot) {
    if (ws.pinned) cudaFreeHost(ws.pinned);
    ws.pinned = nullptr;
    ws.pinned_cap = 0;
    WCK(cudaMallocHost(&ws.pinned, tot));
    ws.pinned_cap = tot;
  }
  {
    size_t off = 0;
    for (const Back& b : back) {
      if (b.bytes) WCK(cudaMemcpyAsync(ws.pinned + off, b.src, b.bytes, cudaMemcpyDeviceToHost, st));
      off += align256(b.bytes);
    }
    WCK(cudaStreamSynchronize(st));
    off = 0;
    for (const Back& b : back) {
      if (b.bytes) std::memcpy(b.dst, ws.pinned + off, b.bytes);
      off += align256(b.bytes);
    }
  }
  return MCBA_OK;
}

void window_release(int device) {
  std::lock_guard<std::mutex> lock(g_win_mutex);
  for (int dv = 0; dv < (int)g_win_ws.size(); ++dv) {
    if (device >= 0 && dv != device) continue;
    WinWorkspace* ws = g_win_ws[dv];
    if (!ws) continue;
    cudaSetDevice(dv);
    if (ws->stream) {
      cudaStreamSynchronize(ws->stream);
      cudaStreamDestroy(ws->stream);
    }
    ws->map.release();
    ws->win.release();
    if (ws->pinned) cudaFreeHost(ws->pinned);
    delete ws;
    g_win_ws[dv] = nullptr;
  }
}

}  // namespace mcba
