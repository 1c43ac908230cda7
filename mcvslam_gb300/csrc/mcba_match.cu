// mcba_match.cu -- brute-force Hamming k = 2 matching of 32-byte descriptors.
//
// Matcher::KnnMatch over descriptor lists (src/Matcher.cpp:245-302) with
// HammingDistance (include/Matcher.hpp:19-31): for each query the best and
// second-best train descriptor, scanned in train order with strict '<', from
// d = {999, 999}, idx = {0, 0}.  That is the two smallest (distance, index)
// pairs in lexicographic order, so the work splits freely and merges
// deterministically to the sequential scan's answer.
//
// Work split: the query x train matrix is cut into tiles of 128 queries x 256
// train descriptors, numbered query-block-major.  A grid of exactly the
// resident CTA count (SMs x CTAs per SM) takes equal contiguous ranges of
// tiles, so every SM carries the same load.  A CTA keeps one running top-2 per
// query (one query per thread, its 32 bytes in registers) while its range
// stays in one query block and writes a partial when the block changes or the
// range ends; partial (cta b, query block g) sits in segment b + g.  A second
// kernel merges, per query, the partials of the CTAs whose ranges touch its
// block, and evaluates the filters the callers apply
// (MatchResKnn::FilterRatio, src/Matcher.cpp:100-111; MatchRes::FilterThreshold,
// src/Matcher.cpp:23-34).
// Inner loop: train tiles staged in shared memory and read as broadcasts; per
// pair 8 XOR, 6 LOP3 of carry-save adders, 5 POPC, a few adds, and the top-2
// of a tile kept as packed (distance << 9 | tile offset) keys with three
// min/max operations.  The population-count pipe (16 per SM per clock) and the
// ALU pipe (64 per SM per clock) bound it about equally; no tensor cores by
// design.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>
#include <vector>

#include "mcba.h"

namespace {

constexpr int kQ = 128;     // queries per CTA (one per thread)
constexpr int kTile = 256;  // train descriptors per tile (8 KB of shared memory)
constexpr unsigned kNone = 999;

struct Top2 {
  unsigned d0, i0, d1, i1;
};

__device__ __forceinline__ bool lex_less(unsigned da, unsigned ia, unsigned db, unsigned ib) {
  return da < db || (da == db && ia < ib);
}

// two smallest of {a0, a1, b0, b1} in (distance, index) order (a0 <= a1, b0 <= b1)
__device__ __forceinline__ Top2 merge2(const Top2& a, const Top2& b) {
  Top2 r;
  if (lex_less(b.d0, b.i0, a.d0, a.i0)) {
    r.d0 = b.d0;
    r.i0 = b.i0;
    const bool bb = lex_less(b.d1, b.i1, a.d0, a.i0);
    r.d1 = bb ? b.d1 : a.d0;
    r.i1 = bb ? b.i1 : a.i0;
  } else {
    r.d0 = a.d0;
    r.i0 = a.i0;
    const bool bb = lex_less(b.d0, b.i0, a.d1, a.i1);
    r.d1 = bb ? b.d0 : a.d1;
    r.i1 = bb ? b.i0 : a.i1;
  }
  return r;
}

// Hamming distance of two 32-byte descriptors.  Three carry-save adders
// (per-bit full adders: popc(x) + popc(y) + popc(z) = popc(x^y^z) +
// 2 popc(maj(x, y, z))) fold seven of the eight XOR words, so the distance
// takes five population counts instead of eight; the XOR / majority terms are
// three-input LOP3s on the ALU pipe, which balances the two pipes.
__device__ __forceinline__ unsigned hamming32(const uint4& a0, const uint4& a1, const uint4& b0, const uint4& b1) {
  const unsigned x0 = a0.x ^ b0.x, x1 = a0.y ^ b0.y, x2 = a0.z ^ b0.z, x3 = a0.w ^ b0.w;
  const unsigned x4 = a1.x ^ b1.x, x5 = a1.y ^ b1.y, x6 = a1.z ^ b1.z, x7 = a1.w ^ b1.w;
  const unsigned s1 = x0 ^ x1 ^ x2, c1 = (x0 & x1) | (x2 & (x0 ^ x1));
  const unsigned s2 = x3 ^ x4 ^ x5, c2 = (x3 & x4) | (x5 & (x3 ^ x4));
  const unsigned s3 = s1 ^ s2 ^ x6, c3 = (s1 & s2) | (x6 & (s1 ^ s2));
  return __popc(s3) + __popc(x7) + 2u * (__popc(c1) + __popc(c2) + __popc(c3));
}

// first CTA whose range [b*T/G, (b+1)*T/G) contains `tile`
__host__ __device__ __forceinline__ int cta_of_tile(long long tile, long long T, int G) {
  return (int)(((tile + 1) * (long long)G - 1) / T);
}

__global__ void __launch_bounds__(kQ) k_knn_partial(const uint4* __restrict__ q, int nq, const uint4* __restrict__ t,
                                                    int nt, int nchunk, long long T, Top2* __restrict__ part) {
  __shared__ uint4 st[2 * kTile];
  const int G = gridDim.x;
  const long long t0 = (long long)blockIdx.x * T / G;
  const long long t1 = (long long)(blockIdx.x + 1) * T / G;
  int g = -1;
  uint4 a0 = make_uint4(0u, 0u, 0u, 0u), a1 = a0;
  Top2 r{kNone, 0u, kNone, 0u};
  for (long long tile = t0; tile < t1; ++tile) {
    const int gq = (int)(tile / nchunk);
    const int base = (int)(tile - (long long)gq * nchunk) * kTile;
    if (gq != g) {
      if (g >= 0) {
        const int i = g * kQ + threadIdx.x;
        if (i < nq) part[(size_t)(blockIdx.x + g) * kQ + threadIdx.x] = r;
      }
      g = gq;
      const int i = g * kQ + threadIdx.x;
      if (i < nq) {
        a0 = q[2 * (size_t)i];
        a1 = q[2 * (size_t)i + 1];
      }
      r = Top2{kNone, 0u, kNone, 0u};
    }
    const int m = min(kTile, nt - base);
    __syncthreads();  // the previous tile's readers are done
    for (int k = threadIdx.x; k < 2 * m; k += kQ) st[k] = t[2 * (size_t)base + k];
    __syncthreads();
    // packed keys: distance (<= 256) above a 9-bit offset within the tile, so
    // the unsigned order is the (distance, index) order
    unsigned k0 = 0xffffffffu, k1 = 0xffffffffu;
    if (m == kTile) {
#pragma unroll 8
      for (int jj = 0; jj < kTile; ++jj) {
        const uint4 b0 = st[2 * jj], b1 = st[2 * jj + 1];
        const unsigned d = hamming32(a0, a1, b0, b1);
        const unsigned key = (d << 9) | (unsigned)jj;
        const unsigned hi = max(key, k0);
        k0 = min(key, k0);
        k1 = min(hi, k1);
      }
    } else {
      for (int jj = 0; jj < m; ++jj) {
        const uint4 b0 = st[2 * jj], b1 = st[2 * jj + 1];
        const unsigned d = hamming32(a0, a1, b0, b1);
        const unsigned key = (d << 9) | (unsigned)jj;
        const unsigned hi = max(key, k0);
        k0 = min(key, k0);
        k1 = min(hi, k1);
      }
    }
    // fold the tile's top-2 into the running one; an empty slot stays (999, 0)
    Top2 tt{kNone, 0u, kNone, 0u};
    if (k0 != 0xffffffffu) {
      tt.d0 = k0 >> 9;
      tt.i0 = (unsigned)base + (k0 & 511u);
    }
    if (k1 != 0xffffffffu) {
      tt.d1 = k1 >> 9;
      tt.i1 = (unsigned)base + (k1 & 511u);
    }
    r = merge2(r, tt);
  }
  if (g >= 0) {
    const int i = g * kQ + threadIdx.x;
    if (i < nq) part[(size_t)(blockIdx.x + g) * kQ + threadIdx.x] = r;
  }
}

__global__ void k_knn_merge(const Top2* __restrict__ part, int nq, int nchunk, long long T, int G, int32_t* idx,
                            int32_t* dist, float ratio, int32_t max_dist, uint8_t* keep) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nq) return;
  const int g = i / kQ, lane = i - g * kQ;
  const int b_lo = cta_of_tile((long long)g * nchunk, T, G);
  const int b_hi = cta_of_tile((long long)(g + 1) * nchunk - 1, T, G);
  Top2 r = part[(size_t)(b_lo + g) * kQ + lane];
  for (int b = b_lo + 1; b <= b_hi; ++b) r = merge2(r, part[(size_t)(b + g) * kQ + lane]);
  idx[2 * (size_t)i] = (int32_t)r.i0;
  idx[2 * (size_t)i + 1] = (int32_t)r.i1;
  dist[2 * (size_t)i] = (int32_t)r.d0;
  dist[2 * (size_t)i + 1] = (int32_t)r.d1;
  if (keep) {
    // the DMatch distances are floats: d0 / d1 <= ratio (0 / 0 gives NaN: dropped)
    const float rr = (float)r.d0 / (float)r.d1;
    keep[i] = (rr <= ratio && (float)r.d0 <= (float)max_dist) ? 1 : 0;
  }
}

// with no train descriptors every query keeps d = {999, 999}, idx = {0, 0}
__global__ void k_knn_empty(int nq, int32_t* idx, int32_t* dist, float ratio, int32_t max_dist, uint8_t* keep) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nq) return;
  idx[2 * (size_t)i] = 0;
  idx[2 * (size_t)i + 1] = 0;
  dist[2 * (size_t)i] = (int32_t)kNone;
  dist[2 * (size_t)i + 1] = (int32_t)kNone;
  if (keep) keep[i] = (1.0f <= ratio && (float)kNone <= (float)max_dist) ? 1 : 0;
}

struct Plan {
  int nchunk;   // train tiles per query block
  long long T;  // tiles in total
  int G;        // CTAs
  size_t part_bytes;
};

// resident CTAs per SM of k_knn_partial, per device
int resident_per_sm(int dev) {
  static std::mutex mu;
  static std::vector<int> cache;
  std::lock_guard<std::mutex> lk(mu);
  if ((int)cache.size() <= dev) cache.resize(dev + 1, 0);
  if (!cache[dev]) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_knn_partial, kQ, 0) != cudaSuccess || n < 1) n = 1;
    cache[dev] = n;
  }
  return cache[dev];
}

Plan plan(int nq, int nt, int dev) {
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  Plan p;
  const int qb = (nq + kQ - 1) / kQ;
  p.nchunk = std::max(1, (nt + kTile - 1) / kTile);
  p.T = (long long)qb * p.nchunk;
  p.G = (int)std::min<long long>(p.T, (long long)sms * resident_per_sm(dev));
  p.part_bytes = (size_t)(p.G + qb) * kQ * sizeof(Top2);
  return p;
}

// per-device scratch for the partials (grown on demand)
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

// part: a buffer of at least plan(...).part_bytes, or null for the cached
// per-device scratch
int launch(const uint8_t* q, int nq, const uint8_t* t, int nt, int32_t* idx, int32_t* dist, float ratio,
           int32_t max_dist, uint8_t* keep, void* part, cudaStream_t st) {
  int dev = 0;
  cudaGetDevice(&dev);
  if (nt == 0) {
    k_knn_empty<<<(nq + 255) / 256, 256, 0, st>>>(nq, idx, dist, ratio, max_dist, keep);
    return cudaGetLastError() == cudaSuccess ? MCBA_OK : MCBA_ERR_CUDA;
  }
  const Plan p = plan(nq, nt, dev);
  if (!part && scratch(dev, p.part_bytes, &part) != cudaSuccess) return MCBA_ERR_NOMEM;
  k_knn_partial<<<p.G, kQ, 0, st>>>(reinterpret_cast<const uint4*>(q), nq, reinterpret_cast<const uint4*>(t), nt,
                                    p.nchunk, p.T, static_cast<Top2*>(part));
  k_knn_merge<<<(nq + 255) / 256, 256, 0, st>>>(static_cast<const Top2*>(part), nq, p.nchunk, p.T, p.G, idx, dist,
                                                 ratio, max_dist, keep);
  return cudaGetLastError() == cudaSuccess ? MCBA_OK : MCBA_ERR_CUDA;
}

}  // namespace

extern "C" int mcba_knn_hamming_device(const uint8_t* query, int32_t nq, const uint8_t* train, int32_t nt,
                                       int32_t* idx, int32_t* dist, float ratio, int32_t max_dist, uint8_t* keep,
                                       void* stream) {
  if (nq < 0 || nt < 0 || (nq > 0 && (!query || !idx || !dist)) || (nt > 0 && !train)) return MCBA_ERR_INVALID;
  if ((reinterpret_cast<uintptr_t>(query) | reinterpret_cast<uintptr_t>(train)) & 15u) return MCBA_ERR_INVALID;
  if (nq == 0) return MCBA_OK;
  return launch(query, nq, train, nt, idx, dist, ratio, max_dist, keep, nullptr, static_cast<cudaStream_t>(stream));
}

extern "C" int mcba_knn_hamming(int32_t device, const uint8_t* query, int32_t nq, const uint8_t* train, int32_t nt,
                                int32_t* idx, int32_t* dist, float ratio, int32_t max_dist, uint8_t* keep,
                                double* ms_device) {
  if (nq < 0 || nt < 0 || (nq > 0 && (!query || !idx || !dist)) || (nt > 0 && !train)) return MCBA_ERR_INVALID;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return MCBA_ERR_NO_DEVICE;
  if (device < 0 || device >= n || cudaSetDevice(device) != cudaSuccess) return MCBA_ERR_INVALID;
  if (ms_device) *ms_device = 0.0;
  if (nq == 0) return MCBA_OK;
  uint8_t *dq = nullptr, *dt = nullptr, *dk = nullptr;
  int32_t *di = nullptr, *dd = nullptr;
  void* dp = nullptr;
  const size_t part_bytes = nt ? plan(nq, nt, device).part_bytes : 16;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int r = MCBA_ERR_CUDA;
  do {
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) break;
    if (cudaMalloc(&dq, 32 * (size_t)nq) != cudaSuccess || cudaMalloc(&dt, 32 * (size_t)std::max(nt, 1)) != cudaSuccess ||
        cudaMalloc(&di, 8 * (size_t)nq) != cudaSuccess || cudaMalloc(&dd, 8 * (size_t)nq) != cudaSuccess ||
        (keep && cudaMalloc(&dk, (size_t)nq) != cudaSuccess) || cudaMalloc(&dp, part_bytes) != cudaSuccess) {
      r = MCBA_ERR_NOMEM;
      break;
    }
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    if (cudaMemcpyAsync(dq, query, 32 * (size_t)nq, cudaMemcpyHostToDevice, st) != cudaSuccess) break;
    if (nt && cudaMemcpyAsync(dt, train, 32 * (size_t)nt, cudaMemcpyHostToDevice, st) != cudaSuccess) break;
    cudaEventRecord(e0, st);
    r = launch(dq, nq, dt, nt, di, dd, ratio, max_dist, dk, dp, st);
    cudaEventRecord(e1, st);
    if (r) break;
    r = MCBA_ERR_CUDA;
    if (cudaMemcpyAsync(idx, di, 8 * (size_t)nq, cudaMemcpyDeviceToHost, st) != cudaSuccess) break;
    if (cudaMemcpyAsync(dist, dd, 8 * (size_t)nq, cudaMemcpyDeviceToHost, st) != cudaSuccess) break;
    if (keep && cudaMemcpyAsync(keep, dk, (size_t)nq, cudaMemcpyDeviceToHost, st) != cudaSuccess) break;
    if (cudaStreamSynchronize(st) != cudaSuccess) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms_device) *ms_device = ms;
    r = MCBA_OK;
  } while (false);
  if (st) cudaStreamSynchronize(st);
  cudaFree(dq);
  cudaFree(dt);
  cudaFree(di);
  cudaFree(dd);
  cudaFree(dk);
  cudaFree(dp);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  return r;
}
