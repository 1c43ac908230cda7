// mcba_chol.cu -- FP64 solve of the reduced camera system on one
// thread-block cluster, launched as its own kernel; the device code is in
// mcba_chol_dev.cuh.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "mcba_chol.h"
#include "mcba_chol_dev.cuh"

namespace mcba {
namespace {
using namespace chold;

__global__ void __launch_bounds__(kThreads, 1) k_ldlt_cluster(const double* S, double* ws, double* x,
                                                              int* solve_ok, Geo g) {
  extern __shared__ __align__(16) double sm[];
  // launched as a programmatic dependent of the Schur assembly: wait for it
  asm volatile("griddepcontrol.wait;" ::: "memory");
  ldlt_cluster_run(S, ws, x, solve_ok, g, sm);
}

}  // namespace

size_t chol_cluster_ws_doubles(int ld, int n) {
  return std::max((size_t)(ld + 32) * ld, make_geo(16, ld, n).ws_doubles());
}

int chol_cluster_plan(int ld, int n, CholPlan* plan) {
  plan->ok = false;
  const int nblk = (n + kB - 1) / kB;
  if (n <= 0 || ld < kB * nblk || nblk > kMaxBlk) return 0;
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
  // cluster size by the work: a chain CTA, the lookahead worker and enough
  // general workers for the trailing updates (small systems, e.g. the
  // windows of a batch that run side by side, take fewer SMs)
  const int Cpref = nblk >= 10 ? 16 : (nblk >= 5 ? 8 : 4);
  for (int C : {16, 8, 4}) {
    if (C > Cpref) continue;
    const Geo g = make_geo(C, ld, n);
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
    plan->smem_bytes = bytes;
    return 1;
  }
  return 0;
}

cudaError_t chol_cluster_launch(const CholPlan& plan, const double* S, double* ws, int ld, int n, double* x,
                                int* solve_ok, cudaStream_t st) {
  const Geo g = make_geo(plan.cluster, ld, n);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(plan.cluster, 1, 1);
  cfg.blockDim = dim3(kThreads, 1, 1);
  cfg.dynamicSmemBytes = plan.smem_bytes;
  cfg.stream = st;
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = plan.cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 2;
  return cudaLaunchKernelEx(&cfg, k_ldlt_cluster, S, ws, x, solve_ok, g);
}

}  // namespace mcba
