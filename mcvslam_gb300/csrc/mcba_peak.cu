// mcba_peak.cu -- measured FP64 FMA rate of the device, the denominator of
// the roofline of the FP64 factorisation kernels (the measured peaks
// cover HBM bandwidth and BF16 tensor throughput only).
//
// Every thread runs kChains independent FMA chains for `iters` steps; the
// grid holds kBlocksPerSM blocks of 256 threads per SM, so each SM
// sub-partition has several warps with independent FMAs in flight.  Timed
// with CUDA events on a private stream after one warm-up launch.

#include <cuda_runtime.h>

#include "mcba.h"

namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;
constexpr int kBlocksPerSM = 4;

__global__ void __launch_bounds__(kThreads) k_fp64_fma(double seed, int iters, double* sink) {
  double a[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) a[c] = seed + threadIdx.x * 1e-3 + c;
  const double m = 0.999999999, q = 1e-12;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) a[c] = fma(a[c], m, q);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += a[c];
  if (s == 12345.678) sink[blockIdx.x] = s;  // keeps the chains live, never true
}

}  // namespace

extern "C" int mcba_fp64_fma_rate(int32_t device, double* gflops) {
  if (!gflops) return MCBA_ERR_INVALID;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return MCBA_ERR_NO_DEVICE;
  if (cudaSetDevice(device) != cudaSuccess) return MCBA_ERR_CUDA;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return MCBA_ERR_CUDA;
  const int blocks = sms * kBlocksPerSM, iters = 4096;
  double* sink = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = MCBA_OK;
  if (cudaMalloc(&sink, sizeof(double) * blocks) != cudaSuccess ||
      cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
      cudaEventCreate(&e1) != cudaSuccess) {
    rc = MCBA_ERR_CUDA;
  } else {
    k_fp64_fma<<<blocks, kThreads, 0, st>>>(1.0, iters, sink);  // warm-up
    float best = 1e30f;
    for (int r = 0; r < 5 && rc == MCBA_OK; ++r) {
      cudaEventRecord(e0, st);
      k_fp64_fma<<<blocks, kThreads, 0, st>>>(1.0 + r, iters, sink);
      cudaEventRecord(e1, st);
      if (cudaStreamSynchronize(st) != cudaSuccess) {
        rc = MCBA_ERR_CUDA;
        break;
      }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms < best) best = ms;
    }
    if (rc == MCBA_OK) {
      const double flops = 2.0 * (double)blocks * kThreads * kChains * iters;
      *gflops = flops / (best * 1e-3) / 1e9;
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  if (sink) cudaFree(sink);
  return rc;
}
