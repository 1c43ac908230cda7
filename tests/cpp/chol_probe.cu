// Test probe for the cluster factorisation: runs k_ldlt_cluster once on a
// host matrix laid out like the solver's S (row stride ld, identity padding
// beyond n, right-hand side in row ld) and returns x, the solve flag and the
// kernel time.  With hold = 1 the workers leave the flag of the first
// right-hand-side panel unreleased, with hold = 2 the flag of the first
// backward-solve inverse (M_0, P_0), so the waits on it run out and the
// solve must report failure instead of hanging.  Built by
// tests/test_chol_gpu.py.
#include "mcba_chol.cu"

#include <cuda_runtime.h>

extern "C" int chol_probe_solve(const double* S_host, int n, int ld, double* x_host, int hold, int* solve_ok,
                                float* ms) {
  using namespace mcba;
  CholPlan plan;
  if (!chol_cluster_plan(ld, n, &plan)) return -1;
  const size_t total = (size_t)(ld + 32) * ld, wtotal = chol_cluster_ws_doubles(ld, n);
  double *S = nullptr, *ws = nullptr, *x = nullptr;
  int* ok = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = 0;
  const int one = 1;
  // every early exit below goes through the frees at the end
  if (cudaMalloc(&S, total * sizeof(double)) != cudaSuccess || cudaMalloc(&ws, wtotal * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&x, (size_t)ld * sizeof(double)) != cudaSuccess || cudaMalloc(&ok, sizeof(int)) != cudaSuccess) {
    rc = -2;
  } else if (cudaMemcpy(S, S_host, total * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
             cudaMemcpy(x, x_host, (size_t)ld * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
             cudaMemcpy(ok, &one, sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess) {
    rc = -5;
  } else if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    rc = -6;
  } else {
    Geo g = make_geo(plan.cluster, ld, n);
    if (hold == 1) g.hold = g.nblk * g.nblk;  // flag of right-hand-side panel (nblk, 0)
    if (hold == 2) g.hold = g.inv_index(0);   // flag of the inverse M_0 and product P_0
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(plan.cluster, 1, 1);
    cfg.blockDim = dim3(kThreads, 1, 1);
    cfg.dynamicSmemBytes = plan.smem_bytes;
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeClusterDimension;
    attr.val.clusterDim.x = plan.cluster;
    attr.val.clusterDim.y = 1;
    attr.val.clusterDim.z = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    cudaEventRecord(e0);
    if (cudaLaunchKernelEx(&cfg, k_ldlt_cluster, (const double*)S, ws, x, ok, g) != cudaSuccess) rc = -3;
    cudaEventRecord(e1);
    if (cudaDeviceSynchronize() != cudaSuccess) rc = -4;
    if (rc == 0 && cudaEventElapsedTime(ms, e0, e1) != cudaSuccess) rc = -7;
    if (rc == 0 && (cudaMemcpy(x_host, x, (size_t)ld * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess ||
                    cudaMemcpy(solve_ok, ok, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess))
      rc = -5;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(S);
  cudaFree(ws);
  cudaFree(x);
  cudaFree(ok);
  return rc;
}
