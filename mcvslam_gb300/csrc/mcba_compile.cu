// mcba_compile.cu -- structure compilation on the device.
//
// The same arrays as compile_structure (mcba_api.cpp), which follows
// SparseOptimizer::initializeOptimization / buildIndexMapping
// (sparse_optimizer.cpp:168-188,201-272) and BlockSolver::buildStructure
// (block_solver.hpp:103-256), built on the GPU from the raw edge list so
// that a new problem costs one upload of its edges instead of a host pass:
//   active set and Hessian numbering   flag kernels + exclusive scans
//   canonical (point-sorted) order     per-point counts, scan, fill, then a
//                                      per-point sort by (pose index, id)
//   pose-sorted stream                 stable multi-way partition by pose
//   Schur pair list                    per-point pair emission in visit
//                                      order, LSD radix passes of the stable
//                                      partition on the block id
// Every ordering is a deterministic function of the input (counts by
// atomics are order independent; ranks come from stable partitions; the
// per-point fill is sorted on unique keys), so the output equals the host
// compilation element for element.
//
// Stable partition: keys in [0, nb), nb <= 1024, tiles of 2048 keys.  A
// histogram per tile (bucket-major) is scanned; inside a tile eight rounds
// of 256 keys rank equal keys with __match_any_sync and per-warp counts, so
// the order of equal keys is kept.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "mcba.h"
#include "mcba_host_pool.h"
#include "mcba_internal.h"

namespace mcba {
namespace {

constexpr int kChunk = 256;       // edges per linearisation chunk (one pose per chunk)
constexpr int kPairChunk = 128;   // Schur pairs per warp task
constexpr int kScanBlock = 1024;  // elements per scan block (256 threads x 4)
constexpr int kPartTile = 2048;   // keys per partition tile (256 threads x 8 rounds)
constexpr int kMaxBuckets = 1024;
constexpr int kRadixBits = 10;

#define CK(call)                                                                   \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess) {                                                       \
      if (err) *err = std::string(#call) + ": " + cudaGetErrorString(e_);          \
      return MCBA_ERR_CUDA;                                                        \
    }                                                                              \
  } while (0)

// ------------------------------------------------------------- scan --
// In place exclusive scan of a[0..n) (the caller's a[n-1] is part of the
// input; the total is written to a[n]).  One level per 1024 elements; a
// single-block scan writes the total itself, and the add pass of a
// multi-block scan copies it from the scanned block sums.
__global__ void __launch_bounds__(256) k_scan_block(int* a, int n, int* sums) {
  __shared__ int warp_tot[8];
  const int base = blockIdx.x * kScanBlock + threadIdx.x * 4;
  int v[4], loc[4], acc = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    v[q] = (base + q < n) ? a[base + q] : 0;
    loc[q] = acc;
    acc += v[q];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int inc = acc;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) warp_tot[warp] = inc;
  __syncthreads();
  int wpre = 0;
  for (int w = 0; w < warp; ++w) wpre += warp_tot[w];
  const int excl = wpre + inc - acc;
#pragma unroll
  for (int q = 0; q < 4; ++q)
    if (base + q < n) a[base + q] = excl + loc[q];
  if (threadIdx.x == 255) {
    sums[blockIdx.x] = wpre + inc;
    if (gridDim.x == 1) a[n] = wpre + inc;
  }
}

__global__ void k_scan_add(int* a, int n, const int* offs) {
  const int i = blockIdx.x * kScanBlock + threadIdx.x;
  const int o = offs[blockIdx.x];
  for (int q = 0; q < kScanBlock; q += 256)
    if (i + q < n) a[i + q] += o;
  if (blockIdx.x == 0 && threadIdx.x == 0) a[n] = offs[gridDim.x];  // the total
}

__global__ void k_add(int* dst, const int* a, const int* b, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = a[i] + b[i];
}

// ------------------------------------------------- stable partition --
__global__ void __launch_bounds__(256) k_part_hist(const int* keys, int n, int nb, int ntiles, int* hist) {
  extern __shared__ int h[];
  for (int b = threadIdx.x; b < nb; b += 256) h[b] = 0;
  __syncthreads();
  const int t0 = blockIdx.x * kPartTile;
  for (int q = 0; q < kPartTile; q += 256) {
    const int i = t0 + q + threadIdx.x;
    if (i < n) atomicAdd(&h[keys[i]], 1);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < nb; b += 256) hist[(size_t)b * ntiles + blockIdx.x] = h[b];
}

// pos[i] = base[k] + (rank of i among the keys equal to k = keys[i]), with
// base = the exclusive prefix of the bucket totals when base is null.
__global__ void __launch_bounds__(256) k_part_scatter(const int* keys, int n, int nb, int ntiles, const int* off,
                                                      const int* base, int* pos) {
  extern __shared__ int sm[];
  int* run = sm;       // [nb] keys of each bucket placed by earlier rounds
  int* wc = sm + nb;   // [8][nb] per-warp counts of the current round
  for (int b = threadIdx.x; b < nb; b += 256) run[b] = 0;
  for (int b = threadIdx.x; b < 8 * nb; b += 256) wc[b] = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  const int tile = blockIdx.x;
  for (int q = 0; q < kPartTile; q += 256) {
    const int i = tile * kPartTile + q + threadIdx.x;
    const bool valid = i < n;
    const int k = valid ? keys[i] : -1 - lane;  // invalid lanes get distinct keys
    const unsigned peers = __match_any_sync(0xffffffffu, k);
    const int rank = __popc(peers & lt);
    const bool leader = (peers & lt) == 0;
    if (valid && leader) wc[warp * nb + k] = __popc(peers);
    __syncthreads();
    if (valid) {
      int pre = 0;
      for (int w = 0; w < warp; ++w) pre += wc[w * nb + k];
      const int t_off = off[(size_t)k * ntiles + tile];
      const int b_off = base ? base[k] + (t_off - off[(size_t)k * ntiles]) : t_off;
      pos[i] = b_off + run[k] + pre + rank;
    }
    __syncthreads();
    if (valid && leader) {
      atomicAdd(&run[k], __popc(peers));
      wc[warp * nb + k] = 0;
    }
    __syncthreads();
  }
}

// atomicAdd(&c[k], 1) with one atomic per distinct key in the warp (callers
// in a warp often hit the same few counters)
__device__ __forceinline__ void count_warp(int* c, int k, bool on) {
  const unsigned m = __ballot_sync(0xffffffffu, on);
  if (!on) return;
  const unsigned peers = __match_any_sync(m, k);
  if ((peers & ((1u << (threadIdx.x & 31)) - 1u)) == 0) atomicAdd(&c[k], __popc(peers));
}

// ------------------------------------------------------ compile kernels --
struct Raw {
  const int* pose;
  const int* point;
  const uint8_t* type;
  const uint8_t* cam;
  const uint8_t* level;
  const uint8_t* robust;
  const float* info;
  const float* delta;
  const float* obs;
  const uint8_t* pose_fixed;
  const uint8_t* point_fixed;
};

// active set (sparse_optimizer.cpp:201-272): level 0 and not all vertices fixed
__global__ void k_mark(Raw r, int E, int* act, int* unary_flag, int* pose_act, int* pt_act) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= E) return;
  const bool unary = r.type[i] == MCBA_EDGE_UNARY;
  const bool pf = r.pose_fixed[r.pose[i]] != 0;
  const bool xf = unary ? true : r.point_fixed[r.point[i]] != 0;
  const bool a = r.level[i] == 0 && !(pf && xf);
  act[i] = a ? 1 : 0;
  unary_flag[i] = unary ? 1 : 0;
  if (a) {
    pose_act[r.pose[i]] = 1;
    if (!unary) pt_act[r.point[i]] = 1;
  }
}

// free-vertex flags into a scan buffer
__global__ void k_free_flags(const int* vact, const uint8_t* fixed, int n, int* flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flag[i] = (vact[i] && !fixed[i]) ? 1 : 0;
}

// Hessian index (-1 when not free) and the free-id list, from the scan
__global__ void k_assign(const int* vact, const uint8_t* fixed, const int* scanned, int n, int* h, int* ids) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const bool f = vact[i] && !fixed[i];
  h[i] = f ? scanned[i] : -1;
  if (f && ids) ids[scanned[i]] = i;
}

// per-edge Hessian indices, canonical membership and the per-point / per-
// bucket counts
__global__ void k_edge_index(Raw r, int E, int Kf, const int* act, const int* pose_h, const int* point_h, int* eph,
                             int* elh, int* pt_cnt, int* bucket_cnt, int* canon_cnt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool in = i < E;
  const int ph = in ? pose_h[r.pose[i]] : -1;
  const int lh = (!in || r.type[i] == MCBA_EDGE_UNARY) ? -1 : point_h[r.point[i]];
  if (in) {
    eph[i] = ph;
    elh[i] = lh;
  }
  const bool a = in && act[i];
  const int b = ph >= 0 ? ph : Kf;
  count_warp(bucket_cnt, b, a);
  count_warp(canon_cnt, b, a && lh >= 0);
  count_warp(pt_cnt, lh, a && lh >= 0);
}

__global__ void k_canon_fill(int E, const int* act, const int* elh, const int* pt_begin, int* fillc, int* canon_id) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= E || !act[i] || elh[i] < 0) return;
  const int l = elh[i];
  canon_id[pt_begin[l] + atomicAdd(&fillc[l], 1)] = i;
}

// the edges of one free point by (pose index, id); fixed poses (-1) first
__global__ void k_canon_sort(int Lf, const int* pt_begin, const int* eph, int* canon_id) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= Lf) return;
  const int b0 = pt_begin[l], b1 = pt_begin[l + 1];
  for (int a = b0 + 1; a < b1; ++a) {
    const int v = canon_id[a];
    const long long kv = ((long long)(eph[v] + 1) << 32) | (unsigned)v;
    int b = a - 1;
    while (b >= b0) {
      const int u = canon_id[b];
      const long long ku = ((long long)(eph[u] + 1) << 32) | (unsigned)u;
      if (ku <= kv) break;
      canon_id[b + 1] = u;
      --b;
    }
    canon_id[b + 1] = v;
  }
}

__global__ void k_canon_out(int Ec, int Kf, const int* canon_id, const int* eph, const int* elh, int* canon_of,
                            int* cph, int* clh, int* key) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= Ec) return;
  const int id = canon_id[e];
  canon_of[id] = e;
  cph[e] = eph[id];
  clh[e] = elh[id];
  key[e] = eph[id] >= 0 ? eph[id] : Kf;
}

// active edges without a free point, in id order (flag for the scan)
__global__ void k_noncanon_flag(int E, const int* act, const int* canon_of, int* flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < E) flag[i] = (act[i] && canon_of[i] < 0) ? 1 : 0;
}

__global__ void k_noncanon_list(int E, int Kf, const int* act, const int* canon_of, const int* scanned,
                                const int* eph, int* ids, int* key) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= E || !act[i] || canon_of[i] >= 0) return;
  const int s = scanned[i];
  ids[s] = i;
  key[s] = eph[i] >= 0 ? eph[i] : Kf;
}

__global__ void k_scatter_ids(int n, const int* ids, const int* pos, int* stream) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) stream[pos[i]] = ids ? ids[i] : i;
}

__global__ void k_scatter_canon(int n, const int* canon_id, const int* pos, int* stream) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) stream[pos[e]] = canon_id[e];
}

__global__ void k_recs(Raw r, int E, int P, const int* stream, const int* unary_slot, const int* eph, const int* elh,
                       const int* canon_of, EdgeRec* recs, float* obs) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= E) return;
  const int id = stream[j];
  const bool unary = r.type[id] == MCBA_EDGE_UNARY;
  EdgeRec rc;
  rc.pose = r.pose[id];
  rc.point = unary ? P + unary_slot[id] : r.point[id];
  rc.pose_h = eph[id];
  rc.point_h = unary ? -1 : elh[id];
  rc.canon = canon_of[id];
  rc.type = r.type[id];
  rc.cam = r.cam[id];
  rc.robust = (r.robust[id] && r.delta[id] > 0.f) ? 1 : 0;
  rc.dim = (rc.type == MCBA_EDGE_STEREO) ? 3 : 2;
  rc.info = r.info[id];
  rc.delta = r.delta[id];
  recs[j] = rc;
  obs[3 * (size_t)j] = r.obs[3 * (size_t)id];
  obs[3 * (size_t)j + 1] = r.obs[3 * (size_t)id + 1];
  obs[3 * (size_t)j + 2] = r.obs[3 * (size_t)id + 2];
}

// chunk counts per pose bucket (scan input)
__global__ void k_chunk_count(int nb, const int* bucket_cnt, int* nch) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < nb) nch[b] = (bucket_cnt[b] + kChunk - 1) / kChunk;
}

__global__ void k_chunks(int Kf, int E, const int* pose_edge_begin, const int* chunk_off, int* chunk_begin,
                         int* chunk_pose, int* pose_chunk_begin) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b > Kf) return;
  const int e0 = pose_edge_begin[b], e1 = pose_edge_begin[b + 1];
  int c = chunk_off[b];
  pose_chunk_begin[b] = c;
  for (int a = e0; a < e1; a += kChunk, ++c) {
    chunk_begin[c] = a;
    chunk_pose[c] = b < Kf ? b : -1;
  }
  if (b == Kf) chunk_begin[chunk_off[Kf + 1]] = E;
}

// canonical edges of every free pose, ascending canonical index: the leading
// part of the pose's stream segment
__global__ void k_pose_canon(int E, int Kf, const int* pose_edge_begin, const int* canon_cnt, const int* pcb,
                             const int* stream, const int* canon_of, int* list) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= E) return;
  int lo = 0, hi = Kf + 1;  // bucket b with pose_edge_begin[b] <= j < pose_edge_begin[b + 1]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (pose_edge_begin[mid] <= j) lo = mid;
    else hi = mid;
  }
  const int b = lo, rr = j - pose_edge_begin[b];
  if (b < Kf && rr < canon_cnt[b]) list[pcb[b] + rr] = canon_of[stream[j]];
}

// pairs of one point in visit order (i before j in canonical order, both
// on free poses; two edges of the point on the same pose also give (j, i))
template <typename F>
__device__ __forceinline__ void visit_pairs(int b0, int b1, const int* cph, F&& fn) {
  for (int i = b0; i < b1; ++i) {
    const int a = cph[i];
    if (a < 0) continue;
    for (int j = i; j < b1; ++j) {
      const int b = cph[j];
      if (b < 0) continue;
      fn(a, b, i, j);
      if (j != i && a == b) fn(a, b, j, i);
    }
  }
}

__global__ void k_pair_count(int Lf, int Kf, const int* pt_begin, const int* cph, int* npairs, int* present) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= Lf) return;
  int c = 0;
  visit_pairs(pt_begin[l], pt_begin[l + 1], cph, [&](int a, int b, int, int) {
    ++c;
    present[a * Kf + b] = 1;
  });
  npairs[l] = c;
}

__global__ void k_diag_present(int Kf, int* present) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a < Kf) present[a * Kf + a] = 1;
}

__global__ void k_block_ids(int Kf, const int* flag_scan, const int* present, int* blk_of, int* block_ab) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= Kf * Kf) return;
  if (present[idx]) {
    const int id = flag_scan[idx];
    blk_of[idx] = id;
    block_ab[2 * id] = idx / Kf;
    block_ab[2 * id + 1] = idx % Kf;
  }
}

// pair counts per block.  When the block counters fit in shared memory each
// CTA counts its points' pairs there and adds one total per block it saw to
// the global counters; otherwise each thread counts its point's pairs per
// block in a short local list first (a point has few distinct pose pairs),
// so the global atomics are one per (point, block).
constexpr int kBlockHistMax = 12288;  // 48 KB of int counters
__global__ void k_pair_block_count(int Lf, int Kf, int nblk, const int* pt_begin, const int* cph, const int* blk_of,
                                   int* bcnt) {
  extern __shared__ int hist[];
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (nblk <= kBlockHistMax) {
    for (int k = threadIdx.x; k < nblk; k += blockDim.x) hist[k] = 0;
    __syncthreads();
    if (l < Lf)
      visit_pairs(pt_begin[l], pt_begin[l + 1], cph, [&](int a, int b, int, int) { atomicAdd(&hist[blk_of[a * Kf + b]], 1); });
    __syncthreads();
    for (int k = threadIdx.x; k < nblk; k += blockDim.x)
      if (hist[k]) atomicAdd(&bcnt[k], hist[k]);
    return;
  }
  if (l >= Lf) return;
  constexpr int kList = 8;
  int key[kList] = {0}, cnt[kList] = {0}, n = 0;
  visit_pairs(pt_begin[l], pt_begin[l + 1], cph, [&](int a, int b, int, int) {
    const int k = blk_of[a * Kf + b];
    int q = 0;
    while (q < n && key[q] != k) ++q;
    if (q < n) {
      ++cnt[q];
    } else if (n < kList) {
      key[n] = k;
      cnt[n] = 1;
      ++n;
    } else {
      atomicAdd(&bcnt[k], 1);
    }
  });
  for (int q = 0; q < n; ++q) atomicAdd(&bcnt[key[q]], cnt[q]);
}

__global__ void k_pchunk_count(int nblk, const int* bcnt, int* nch) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < nblk) nch[k] = (bcnt[k] + kPairChunk - 1) / kPairChunk;
}

__global__ void k_pair_emit(int Lf, int Kf, const int* pt_begin, const int* cph, const int* blk_of,
                            const int* pair_base, int* key, int2* val) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= Lf) return;
  int v = pair_base[l];
  visit_pairs(pt_begin[l], pt_begin[l + 1], cph, [&](int a, int b, int i, int j) {
    key[v] = blk_of[a * Kf + b];
    val[v] = make_int2(i, j);
    ++v;
  });
}

__global__ void k_digit(int n, const int* key, int shift, int* dig) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dig[i] = (key[i] >> shift) & ((1 << kRadixBits) - 1);
}

__global__ void k_permute(int n, const int* pos, const int* key, const int2* val, int* key2, int2* val2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  key2[pos[i]] = key[i];
  val2[pos[i]] = val[i];
}

__global__ void k_pchunks(int nblk, int npairs, const int* boff, const int* bcb, int* pchunk_begin) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nblk) return;
  int c = bcb[k];
  for (int a = boff[k]; a < boff[k + 1]; a += kPairChunk, ++c) pchunk_begin[c] = a;
  if (k == nblk - 1) pchunk_begin[bcb[nblk]] = npairs;
}

inline int blocks(int n, int t = 256) { return std::max(1, (n + t - 1) / t); }

}  // namespace

// One staging-copy task: bytes [b, e) of raw array a.
struct Piece {
  int a;
  size_t b, e;
};

class DeviceCompiler {
 public:
  char* h_stage = nullptr;  // pinned staging of the raw graph
  size_t h_cap = 0;
  int* h_sizes = nullptr;   // pinned
  std::vector<Piece> pieces;  // staging copy tasks (kept for their capacity)
  DBuf<char> d_raw;
  Raw raw{};
  int Eall = 0, K = 0, P = 0, U = 0, Kf = 0, Lf = 0, E = 0, Ec = 0, nchunk = 0, npairs = 0, nblk = 0, npc = 0;
  DBuf<int> act, unary_scan, pose_act, pt_act, pose_scan, pt_scan, pose_h, point_h, eph, elh, pt_begin, fillc,
      bucket_cnt, canon_cnt, pe_begin, nch, pcb, canon_id, canon_of, cph, clh, ckey, npairs_l, present, blk_id,
      blk_of, block_ab, bcnt, bcb, stream, pos, nc_scan, nc_ids, nc_key, base2, pkey, pkey2, pdig, scan_tmp, hist;
  DBuf<int2> pval, pval2;

  ~DeviceCompiler() {
    if (h_stage) cudaFreeHost(h_stage);
    if (h_sizes) cudaFreeHost(h_sizes);
    DBuf<int>* all[] = {&act,      &unary_scan, &pose_act, &pt_act,     &pose_scan, &pt_scan, &pose_h,  &point_h,
                        &eph,      &elh,        &pt_begin, &fillc,      &bucket_cnt, &canon_cnt, &pe_begin, &nch,
                        &pcb,      &canon_id,   &canon_of, &cph,        &clh,       &ckey,    &npairs_l, &present,
                        &blk_id,   &blk_of,     &block_ab, &bcnt,       &bcb,       &stream,  &pos,     &nc_scan,
                        &nc_ids,   &nc_key,     &base2,    &pkey,       &pkey2,     &pdig,    &scan_tmp, &hist};
    for (auto* b : all) b->release();
    pval.release();
    pval2.release();
    d_raw.release();
  }

  static size_t scan_tmp_need(int n) {
    size_t t = 2;
    while (n > 1) {
      n = (n + kScanBlock - 1) / kScanBlock;
      t += (size_t)n + 1;
    }
    return t;
  }

  // exclusive scan of a[0..n) in place; the total goes to a[n]
  int scan(int* a, int n, cudaStream_t st, std::string* err, size_t tmp_off = 0) {
    if (n <= 0) {
      CK(cudaMemsetAsync(a, 0, sizeof(int), st));
      return MCBA_OK;
    }
    if (tmp_off == 0) CK(scan_tmp.ensure(scan_tmp_need(n)));
    const int nb = (n + kScanBlock - 1) / kScanBlock;
    int* sums = scan_tmp.p + tmp_off;  // [nb + 1]
    k_scan_block<<<nb, 256, 0, st>>>(a, n, sums);
    if (nb == 1) {
      CK(cudaGetLastError());
      return MCBA_OK;
    }
    const int r = scan(sums, nb, st, err, tmp_off + nb + 1);
    if (r) return r;
    k_scan_add<<<nb, 256, 0, st>>>(a, n, sums);
    CK(cudaGetLastError());
    return MCBA_OK;
  }

  // stable partition of keys[0..n) (values in [0, nb)); see k_part_scatter
  int partition(const int* keys, int n, int nb, const int* base, int* out_pos, cudaStream_t st, std::string* err) {
    if (n <= 0) return MCBA_OK;
    const int ntiles = (n + kPartTile - 1) / kPartTile;
    const int hn = nb * ntiles;
    CK(hist.ensure((size_t)hn + 1));
    k_part_hist<<<ntiles, 256, nb * sizeof(int), st>>>(keys, n, nb, ntiles, hist.p);
    const int r = scan(hist.p, hn, st, err);
    if (r) return r;
    k_part_scatter<<<ntiles, 256, 9 * nb * sizeof(int), st>>>(keys, n, nb, ntiles, hist.p, base, out_pos);
    CK(cudaGetLastError());
    return MCBA_OK;
  }

  int read(int* dst_host_slot, const int* src, cudaStream_t st, std::string* err) {
    CK(cudaMemcpyAsync(dst_host_slot, src, sizeof(int), cudaMemcpyDeviceToHost, st));
    return MCBA_OK;
  }
};

DeviceCompiler* compiler_create() { return new DeviceCompiler(); }
void compiler_destroy(DeviceCompiler* c) { delete c; }

int compiler_phase1(DeviceCompiler* c, const HostProblem& hp, cudaStream_t st, StructureSizes* sz, int64_t* h2d,
                    std::string* err) {
  const int Eall = (int)hp.n_edges(), K = (int)hp.poses.size(), P = (int)hp.point_fixed.size();
  if ((int64_t)Eall * 16 >= ((int64_t)1 << 31) || K >= kMaxBuckets) {
    if (err) *err = "problem above the device structure compiler's range";
    return MCBA_ERR_TOO_LARGE;
  }
  c->Eall = Eall;
  c->K = K;
  c->P = P;
  // ---- raw graph: one pinned staging area, one copy
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t n8 = (size_t)Eall;
  const size_t sizes[11] = {4 * n8, 4 * n8, n8, n8, n8, n8, 4 * n8, 4 * n8, 12 * n8, (size_t)K, (size_t)P};
  size_t off[11], cur = 0;
  for (int i = 0; i < 11; ++i) {
    off[i] = cur;
    cur = al(cur + sizes[i]);
  }
  if (cur > c->h_cap) {
    if (c->h_stage) cudaFreeHost(c->h_stage);
    c->h_stage = nullptr;
    c->h_cap = 0;
    CK(cudaMallocHost(&c->h_stage, cur));
    c->h_cap = cur;
  }
  if (!c->h_sizes) CK(cudaMallocHost(&c->h_sizes, 16 * sizeof(int)));
  char* h = c->h_stage;
  // the staging copies in pieces of at most 128 KB spread over the host
  // pool (one array per task left the 12-byte observations on one thread,
  // the longest task by far); the camera indices are narrowed to bytes
  const void* src[11] = {hp.e_pose.data(),  hp.e_point.data(), hp.e_type.data(),  nullptr,
                         hp.e_level.data(), hp.e_robust.data(), hp.e_info.data(), hp.e_delta.data(),
                         hp.e_obs.data(),   hp.pose_fixed.data(), hp.point_fixed.data()};
  constexpr size_t kPiece = 128 * 1024;
  std::vector<Piece>& pieces = c->pieces;
  pieces.clear();
  for (int a = 0; a < 11; ++a) {
    if (a < 9 && !Eall) continue;
    const size_t n = sizes[a];  // bytes (for the camera indices: bytes of the output)
    for (size_t b = 0; b < n; b += kPiece) pieces.push_back(Piece{a, b, std::min(n, b + kPiece)});
  }
  HostPool::get().run((int)pieces.size(), [&](int t) {
    const Piece& q = pieces[t];
    if (q.a == 3) {
      uint8_t* cam8 = reinterpret_cast<uint8_t*>(h + off[3]);
      for (size_t i = q.b; i < q.e; ++i) cam8[i] = (uint8_t)hp.e_cam[i];
    } else {
      std::memcpy(h + off[q.a] + q.b, static_cast<const char*>(src[q.a]) + q.b, q.e - q.b);
    }
  });
  CK(c->d_raw.ensure(cur));
  CK(cudaMemcpyAsync(c->d_raw.p, h, cur, cudaMemcpyHostToDevice, st));
  if (h2d) *h2d += (int64_t)cur;
  char* d = c->d_raw.p;
  Raw& r = c->raw;
  r.pose = (const int*)(d + off[0]);
  r.point = (const int*)(d + off[1]);
  r.type = (const uint8_t*)(d + off[2]);
  r.cam = (const uint8_t*)(d + off[3]);
  r.level = (const uint8_t*)(d + off[4]);
  r.robust = (const uint8_t*)(d + off[5]);
  r.info = (const float*)(d + off[6]);
  r.delta = (const float*)(d + off[7]);
  r.obs = (const float*)(d + off[8]);
  r.pose_fixed = (const uint8_t*)(d + off[9]);
  r.point_fixed = (const uint8_t*)(d + off[10]);
  int rc;

  // ---- active set, unary slots, Hessian numbering
  const size_t E1 = n8 + 1;
  CK(c->act.ensure(E1));
  CK(c->unary_scan.ensure(E1));
  CK(c->pose_act.ensure(K + 1));
  CK(c->pt_act.ensure(P + 1));
  CK(c->pose_scan.ensure(K + 1));
  CK(c->pt_scan.ensure(P + 1));
  CK(c->pose_h.ensure(K + 1));
  CK(c->point_h.ensure(P + 1));
  CK(cudaMemsetAsync(c->pose_act.p, 0, (K + 1) * sizeof(int), st));
  CK(cudaMemsetAsync(c->pt_act.p, 0, (P + 1) * sizeof(int), st));
  if (Eall) k_mark<<<blocks(Eall), 256, 0, st>>>(r, Eall, c->act.p, c->unary_scan.p, c->pose_act.p, c->pt_act.p);
  if ((rc = c->scan(c->unary_scan.p, Eall, st, err))) return rc;
  if (K) k_free_flags<<<blocks(K), 256, 0, st>>>(c->pose_act.p, r.pose_fixed, K, c->pose_scan.p);
  if ((rc = c->scan(c->pose_scan.p, K, st, err))) return rc;
  if (P) k_free_flags<<<blocks(P), 256, 0, st>>>(c->pt_act.p, r.point_fixed, P, c->pt_scan.p);
  if ((rc = c->scan(c->pt_scan.p, P, st, err))) return rc;
  if (K) k_assign<<<blocks(K), 256, 0, st>>>(c->pose_act.p, r.pose_fixed, c->pose_scan.p, K, c->pose_h.p, nullptr);
  if (P) k_assign<<<blocks(P), 256, 0, st>>>(c->pt_act.p, r.point_fixed, c->pt_scan.p, P, c->point_h.p, nullptr);
  if ((rc = c->read(c->h_sizes + 0, c->pose_scan.p + K, st, err))) return rc;
  if ((rc = c->read(c->h_sizes + 1, c->pt_scan.p + P, st, err))) return rc;
  if ((rc = c->read(c->h_sizes + 2, c->unary_scan.p + Eall, st, err))) return rc;
  CK(cudaStreamSynchronize(st));
  const int Kf = c->Kf = c->h_sizes[0];
  const int Lf = c->Lf = c->h_sizes[1];
  c->U = c->h_sizes[2];
  const int nbk = Kf + 1;  // pose buckets: free poses in order, then the fixed-pose edges

  // ---- per-edge indices, canonical order, pose buckets
  CK(c->eph.ensure(E1));
  CK(c->elh.ensure(E1));
  CK(c->pt_begin.ensure(Lf + 1));
  CK(c->fillc.ensure(Lf + 1));
  CK(c->bucket_cnt.ensure(nbk + 1));
  CK(c->canon_cnt.ensure(nbk + 1));
  CK(cudaMemsetAsync(c->pt_begin.p, 0, (Lf + 1) * sizeof(int), st));
  CK(cudaMemsetAsync(c->fillc.p, 0, (Lf + 1) * sizeof(int), st));
  CK(cudaMemsetAsync(c->bucket_cnt.p, 0, (nbk + 1) * sizeof(int), st));
  CK(cudaMemsetAsync(c->canon_cnt.p, 0, (nbk + 1) * sizeof(int), st));
  if (Eall)
    k_edge_index<<<blocks(Eall), 256, 0, st>>>(r, Eall, Kf, c->act.p, c->pose_h.p, c->point_h.p, c->eph.p, c->elh.p,
                                               c->pt_begin.p, c->bucket_cnt.p, c->canon_cnt.p);
  if ((rc = c->scan(c->pt_begin.p, Lf, st, err))) return rc;
  CK(c->canon_id.ensure(E1));
  if (Eall)
    k_canon_fill<<<blocks(Eall), 256, 0, st>>>(Eall, c->act.p, c->elh.p, c->pt_begin.p, c->fillc.p, c->canon_id.p);
  if (Lf) k_canon_sort<<<blocks(Lf, 128), 128, 0, st>>>(Lf, c->pt_begin.p, c->eph.p, c->canon_id.p);
  CK(c->pe_begin.ensure(nbk + 1));
  CK(cudaMemcpyAsync(c->pe_begin.p, c->bucket_cnt.p, nbk * sizeof(int), cudaMemcpyDeviceToDevice, st));
  if ((rc = c->scan(c->pe_begin.p, nbk, st, err))) return rc;
  CK(c->nch.ensure(nbk + 1));
  k_chunk_count<<<blocks(nbk), 256, 0, st>>>(nbk, c->bucket_cnt.p, c->nch.p);
  if ((rc = c->scan(c->nch.p, nbk, st, err))) return rc;
  CK(c->pcb.ensure(Kf + 1));
  if (Kf) CK(cudaMemcpyAsync(c->pcb.p, c->canon_cnt.p, Kf * sizeof(int), cudaMemcpyDeviceToDevice, st));
  if ((rc = c->scan(c->pcb.p, Kf, st, err))) return rc;
  if ((rc = c->read(c->h_sizes + 3, c->pt_begin.p + Lf, st, err))) return rc;
  if ((rc = c->read(c->h_sizes + 4, c->pe_begin.p + nbk, st, err))) return rc;
  if ((rc = c->read(c->h_sizes + 5, c->nch.p + nbk, st, err))) return rc;
  CK(cudaStreamSynchronize(st));
  const int Ec = c->Ec = c->h_sizes[3];
  c->E = c->h_sizes[4];
  c->nchunk = c->h_sizes[5];

  // ---- canonical outputs and the Schur pair structure
  CK(c->canon_of.ensure(E1));
  CK(c->cph.ensure((size_t)Ec + 1));
  CK(c->clh.ensure((size_t)Ec + 1));
  CK(c->ckey.ensure((size_t)Ec + 1));
  CK(cudaMemsetAsync(c->canon_of.p, 0xff, E1 * sizeof(int), st));
  if (Ec)
    k_canon_out<<<blocks(Ec), 256, 0, st>>>(Ec, Kf, c->canon_id.p, c->eph.p, c->elh.p, c->canon_of.p, c->cph.p,
                                            c->clh.p, c->ckey.p);
  const size_t KK = (size_t)Kf * Kf;
  CK(c->npairs_l.ensure(Lf + 1));
  CK(c->present.ensure(KK + 1));
  CK(c->blk_id.ensure(KK + 1));
  CK(cudaMemsetAsync(c->present.p, 0, (KK + 1) * sizeof(int), st));
  if (Lf) k_pair_count<<<blocks(Lf, 128), 128, 0, st>>>(Lf, Kf, c->pt_begin.p, c->cph.p, c->npairs_l.p, c->present.p);
  if (Kf) k_diag_present<<<blocks(Kf), 256, 0, st>>>(Kf, c->present.p);
  CK(cudaMemcpyAsync(c->blk_id.p, c->present.p, KK * sizeof(int), cudaMemcpyDeviceToDevice, st));
  if ((rc = c->scan(c->blk_id.p, (int)KK, st, err))) return rc;
  if ((rc = c->scan(c->npairs_l.p, Lf, st, err))) return rc;
  if ((rc = c->read(c->h_sizes + 6, c->blk_id.p + KK, st, err))) return rc;
  if ((rc = c->read(c->h_sizes + 7, c->npairs_l.p + Lf, st, err))) return rc;
  CK(cudaStreamSynchronize(st));
  const int nblk = c->nblk = c->h_sizes[6];
  c->npairs = c->h_sizes[7];
  CK(c->blk_of.ensure(KK + 1));
  CK(c->block_ab.ensure(2 * (size_t)nblk + 2));
  CK(c->bcnt.ensure(nblk + 1));
  CK(c->bcb.ensure(nblk + 1));
  CK(cudaMemsetAsync(c->bcnt.p, 0, (nblk + 1) * sizeof(int), st));
  if (KK) k_block_ids<<<blocks((int)KK), 256, 0, st>>>(Kf, c->blk_id.p, c->present.p, c->blk_of.p, c->block_ab.p);
  if (Lf) {
    const size_t hist = nblk <= kBlockHistMax ? (size_t)nblk * sizeof(int) : 0;
    k_pair_block_count<<<blocks(Lf, 256), 256, hist, st>>>(Lf, Kf, nblk, c->pt_begin.p, c->cph.p, c->blk_of.p,
                                                            c->bcnt.p);
  }
  if (nblk) k_pchunk_count<<<blocks(nblk), 256, 0, st>>>(nblk, c->bcnt.p, c->bcb.p);
  if ((rc = c->scan(c->bcb.p, nblk, st, err))) return rc;   // block_chunk_begin; npc at [nblk]
  if ((rc = c->scan(c->bcnt.p, nblk, st, err))) return rc;  // pair offset of each block
  if ((rc = c->read(c->h_sizes + 8, c->bcb.p + nblk, st, err))) return rc;
  CK(cudaStreamSynchronize(st));
  c->npc = c->h_sizes[8];
  sz->K = K;
  sz->P = P;
  sz->U = c->U;
  sz->Kf = Kf;
  sz->Lf = Lf;
  sz->E = c->E;
  sz->Ec = Ec;
  sz->nchunk = c->nchunk;
  sz->npairs = c->npairs;
  sz->nblk = nblk;
  sz->npc = c->npc;
  return MCBA_OK;
}

int compiler_phase2(DeviceCompiler* c, const DeviceStructureOut& o, cudaStream_t st, std::string* err) {
  const int Eall = c->Eall, K = c->K, P = c->P, Kf = c->Kf, Lf = c->Lf, E = c->E, Ec = c->Ec;
  const int nblk = c->nblk, npairs = c->npairs, nbk = Kf + 1;
  const Raw& r = c->raw;
  const size_t E1 = (size_t)Eall + 1;
  int rc;
  // free-vertex lists and the arrays phase 1 already holds
  if (K) k_assign<<<blocks(K), 256, 0, st>>>(c->pose_act.p, r.pose_fixed, c->pose_scan.p, K, c->pose_h.p, o.free_pose_ids);
  if (P) k_assign<<<blocks(P), 256, 0, st>>>(c->pt_act.p, r.point_fixed, c->pt_scan.p, P, c->point_h.p, o.free_point_ids);
  CK(cudaMemcpyAsync(o.pt_begin, c->pt_begin.p, (Lf + 1) * sizeof(int), cudaMemcpyDeviceToDevice, st));
  if (Ec) {
    CK(cudaMemcpyAsync(o.canon_pose_h, c->cph.p, Ec * sizeof(int), cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(o.canon_point_h, c->clh.p, Ec * sizeof(int), cudaMemcpyDeviceToDevice, st));
  }
  CK(cudaMemcpyAsync(o.pose_canon_begin, c->pcb.p, (Kf + 1) * sizeof(int), cudaMemcpyDeviceToDevice, st));
  if (nblk) {
    CK(cudaMemcpyAsync(o.block_ab, c->block_ab.p, 2 * (size_t)nblk * sizeof(int), cudaMemcpyDeviceToDevice, st));
  }
  CK(cudaMemcpyAsync(o.block_chunk_begin, c->bcb.p, (nblk + 1) * sizeof(int), cudaMemcpyDeviceToDevice, st));

  // pose-sorted stream: per bucket the canonical edges in canonical order,
  // then the edges without a free point in id order
  CK(c->stream.ensure(E1));
  CK(c->pos.ensure(E1));
  if ((rc = c->partition(c->ckey.p, Ec, nbk, c->pe_begin.p, c->pos.p, st, err))) return rc;
  if (Ec) k_scatter_canon<<<blocks(Ec), 256, 0, st>>>(Ec, c->canon_id.p, c->pos.p, c->stream.p);
  const int nnc = E - Ec;
  if (nnc > 0) {
    CK(c->nc_scan.ensure(E1));
    CK(c->nc_ids.ensure((size_t)nnc + 1));
    CK(c->nc_key.ensure((size_t)nnc + 1));
    CK(c->base2.ensure(nbk + 1));
    k_noncanon_flag<<<blocks(Eall), 256, 0, st>>>(Eall, c->act.p, c->canon_of.p, c->nc_scan.p);
    if ((rc = c->scan(c->nc_scan.p, Eall, st, err))) return rc;
    k_noncanon_list<<<blocks(Eall), 256, 0, st>>>(Eall, Kf, c->act.p, c->canon_of.p, c->nc_scan.p, c->eph.p,
                                                  c->nc_ids.p, c->nc_key.p);
    k_add<<<blocks(nbk), 256, 0, st>>>(c->base2.p, c->pe_begin.p, c->canon_cnt.p, nbk);
    if ((rc = c->partition(c->nc_key.p, nnc, nbk, c->base2.p, c->pos.p, st, err))) return rc;
    k_scatter_ids<<<blocks(nnc), 256, 0, st>>>(nnc, c->nc_ids.p, c->pos.p, c->stream.p);
  }
  if (E) k_recs<<<blocks(E), 256, 0, st>>>(r, E, P, c->stream.p, c->unary_scan.p, c->eph.p, c->elh.p, c->canon_of.p,
                                           o.recs, o.obs);
  k_chunks<<<blocks(nbk), 256, 0, st>>>(Kf, E, c->pe_begin.p, c->nch.p, o.chunk_begin, o.chunk_pose,
                                        o.pose_chunk_begin);
  if (Kf && E)
    k_pose_canon<<<blocks(E), 256, 0, st>>>(E, Kf, c->pe_begin.p, c->canon_cnt.p, c->pcb.p, c->stream.p,
                                            c->canon_of.p, o.pose_canon_list);

  // Schur pairs: emitted in visit order, then stably sorted by block id
  if (npairs > 0) {
    CK(c->pkey.ensure(npairs));
    CK(c->pkey2.ensure(npairs));
    CK(c->pdig.ensure(npairs));
    CK(c->pval.ensure(npairs));
    CK(c->pval2.ensure(npairs));
    CK(c->pos.ensure(std::max<size_t>(E1, npairs)));
    k_pair_emit<<<blocks(Lf, 128), 128, 0, st>>>(Lf, Kf, c->pt_begin.p, c->cph.p, c->blk_of.p, c->npairs_l.p,
                                                 c->pkey.p, c->pval.p);
    int* kin = c->pkey.p;
    int* kout = c->pkey2.p;
    int2* vin = c->pval.p;
    int2* vout = c->pval2.p;
    for (int shift = 0; (nblk - 1) >> shift; shift += kRadixBits) {
      const int nb = std::min(1 << kRadixBits, ((nblk - 1) >> shift) + 1);
      k_digit<<<blocks(npairs), 256, 0, st>>>(npairs, kin, shift, c->pdig.p);
      if ((rc = c->partition(c->pdig.p, npairs, nb, nullptr, c->pos.p, st, err))) return rc;
      k_permute<<<blocks(npairs), 256, 0, st>>>(npairs, c->pos.p, kin, vin, kout, vout);
      std::swap(kin, kout);
      std::swap(vin, vout);
    }
    CK(cudaMemcpyAsync(o.pairs, vin, (size_t)npairs * sizeof(int2), cudaMemcpyDeviceToDevice, st));
  }
  if (nblk) k_pchunks<<<blocks(nblk), 256, 0, st>>>(nblk, npairs, c->bcnt.p, c->bcb.p, o.pchunk_begin);
  else CK(cudaMemsetAsync(o.pchunk_begin, 0, sizeof(int), st));
  CK(cudaGetLastError());
  return MCBA_OK;
}

}  // namespace mcba
