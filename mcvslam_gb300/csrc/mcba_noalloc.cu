// mcba_noalloc.cu -- robust reprojection cost of a batch of mono edges that
// allocates no memory.
//
// Some callers cannot call cudaMalloc: a tracking thread with a hard per-frame
// deadline (cudaMalloc and cudaFree may wait for the whole device to go idle
// and take milliseconds), or a host application that hands the entire device
// memory to its own pool at start-up and does not let libraries allocate
// afterwards.  For them this entry point keeps its scratch -- one partial sum
// per thread block -- in a fixed file-scope device array instead of a
// library allocation.  The caller passes inputs and the output.
//
// The array is sized for kNoAllocMaxBlocks blocks of kNoAllocThreads edges,
// i.e. at most MCBA_NOALLOC_MAX_EDGES edges per call; larger calls are
// rejected.  Every GPU that loads the library holds the 32 KB array until the
// process exits.  All calls on a device share it and it keeps the last call's
// contents: each call first writes every slot it later reads, so nothing has
// to start at zero, but calls whose kernels overlap on the GPU (two streams,
// two host threads) race on the array and must be serialised by the caller.
//
// Host code may not hand the array's name to a kernel: on the host it is a
// stand-in symbol, not a device address.  The first call on each device looks
// up the real address with cudaGetSymbolAddress (with that device current) and
// caches it; make that first call before any stream capture on the device.
// The cached address belongs to the device's context at that time: after a
// cudaDeviceReset of a device, no further call may be made on that device in
// the same process (the array is reloaded at a new address the cache does not
// know).
//
// Error reporting: a CUDA error already pending on the calling thread when the
// call starts is left in place and the call returns MCBA_ERR_CUDA without
// launching; otherwise each launch is checked on its own.

#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "mcba.h"

namespace {

constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocMaxBlocks = MCBA_NOALLOC_MAX_EDGES / kNoAllocThreads;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_cost_partials[kNoAllocMaxBlocks];

double* g_partials_addr[kMaxDevices] = {nullptr};
std::mutex g_setup_mutex;

__device__ __forceinline__ void rot_of_qt(const double* q, double* M) {
  const double x = q[0], y = q[1], z = q[2], w = q[3];
  const double tx = 2 * x, ty = 2 * y, tz = 2 * z;
  M[0] = 1 - (ty * y + tz * z);
  M[1] = ty * x - tz * w;
  M[2] = tz * x + ty * w;
  M[3] = ty * x + tz * w;
  M[4] = 1 - (tx * x + tz * z);
  M[5] = tz * y - tx * w;
  M[6] = tz * x - ty * w;
  M[7] = tz * y + tx * w;
  M[8] = 1 - (tx * x + ty * y);
}

// Per-block partial of sum rho(e' Omega e) (activeRobustChi2,
// sparse_optimizer.cpp:102-116) over mono edges e = obs - pi(T_cb T_bw X).
__global__ void __launch_bounds__(kNoAllocThreads)
    k_cost_partials_noalloc(int64_t n, const double* pose_qt, const double* ext_qt, const double* X, const double* K,
                            const double* obs, const double* info, const double* delta, const uint8_t* robust,
                            double* partials) {
  __shared__ double sh[kNoAllocThreads / 32];
  const int64_t i = blockIdx.x * (int64_t)kNoAllocThreads + threadIdx.x;
  double rho = 0.0;
  if (i < n) {
    double Rb[9], Rc[9];
    rot_of_qt(pose_qt + 7 * i, Rb);
    rot_of_qt(ext_qt + 7 * i, Rc);
    const double* tb = pose_qt + 7 * i + 4;
    const double* tc = ext_qt + 7 * i + 4;
    const double* x = X + 3 * i;
    double Pb[3], Pc[3];
    for (int r = 0; r < 3; ++r) Pb[r] = Rb[3 * r] * x[0] + Rb[3 * r + 1] * x[1] + Rb[3 * r + 2] * x[2] + tb[r];
    for (int r = 0; r < 3; ++r) Pc[r] = Rc[3 * r] * Pb[0] + Rc[3 * r + 1] * Pb[1] + Rc[3 * r + 2] * Pb[2] + tc[r];
    const double* k = K + 4 * i;
    const double e0 = obs[2 * i] - (k[0] * Pc[0] / Pc[2] + k[2]);
    const double e1 = obs[2 * i + 1] - (k[1] * Pc[1] / Pc[2] + k[3]);
    const double om = info ? info[i] : 1.0;
    const double e2 = e0 * (om * e0) + e1 * (om * e1);
    const bool rb = robust ? robust[i] != 0 : true;
    const double d = delta ? delta[i] : 0.0;
    if (rb && d > 0.0) {
      const double dsqr = d * d;
      rho = (e2 <= dsqr) ? e2 : 2.0 * sqrt(e2) * d - dsqr;
    } else {
      rho = e2;
    }
  }
  for (int o = 16; o >= 1; o >>= 1) rho += __shfl_xor_sync(0xffffffffu, rho, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = rho;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < kNoAllocThreads / 32; ++w) s += sh[w];
    partials[blockIdx.x] = s;
  }
}

// Fixed-order sum of the block partials written above by this same call.
__global__ void __launch_bounds__(256) k_cost_total_noalloc(const double* partials, int nblocks, double* out) {
  __shared__ double sh[8];
  double s = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += 256) s += partials[b];
  for (int o = 16; o >= 1; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += sh[w];
    *out = t;
  }
}

// Device address of the scratch array on the current device, looked up once
// per device.
int partials_address(double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return MCBA_ERR_NO_DEVICE;
  if (dev < 0 || dev >= kMaxDevices) return MCBA_ERR_TOO_LARGE;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_partials_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_cost_partials);
    if (e != cudaSuccess || !p) return MCBA_ERR_CUDA;
    g_partials_addr[dev] = static_cast<double*>(p);
  }
  *out = g_partials_addr[dev];
  return MCBA_OK;
}

}  // namespace

extern "C" int mcba_robust_cost_noalloc(int64_t n, const double* pose_qt, const double* ext_qt, const double* X,
                                        const double* K, const double* obs, const double* info, const double* delta,
                                        const uint8_t* robust, double* cost, void* stream) {
  if (n < 0 || !cost) return MCBA_ERR_INVALID;
  if (n > MCBA_NOALLOC_MAX_EDGES) return MCBA_ERR_TOO_LARGE;
  if (n > 0 && (!pose_qt || !ext_qt || !X || !K || !obs)) return MCBA_ERR_INVALID;
  // an error left by an earlier, unrelated call stays with the caller
  if (cudaPeekAtLastError() != cudaSuccess) return MCBA_ERR_CUDA;
  double* partials = nullptr;
  const int r = partials_address(&partials);
  if (r != MCBA_OK) return r;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int nblocks = (int)((n + kNoAllocThreads - 1) / kNoAllocThreads);
  if (nblocks > 0) {
    k_cost_partials_noalloc<<<nblocks, kNoAllocThreads, 0, st>>>(n, pose_qt, ext_qt, X, K, obs, info, delta, robust,
                                                                 partials);
    if (cudaGetLastError() != cudaSuccess) return MCBA_ERR_CUDA;
  }
  k_cost_total_noalloc<<<1, 256, 0, st>>>(partials, nblocks, cost);
  if (cudaGetLastError() != cudaSuccess) return MCBA_ERR_CUDA;
  return MCBA_OK;
}
