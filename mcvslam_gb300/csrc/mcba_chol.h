// mcba_chol.h -- cluster Cholesky solve of the reduced camera system.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace mcba {

struct CholPlan {
  bool ok = false;
  int cluster = 0;
  size_t smem_bytes = 0;
};

// Chooses a cluster size (16, 8 or 4 CTAs by the size) for the n x n system
// (row stride ld); returns 0 (plan.ok = false) when the system is too large
// for the cluster solve.
int chol_cluster_plan(int ld, int n, CholPlan* plan);

// Doubles of the workspace chol_cluster_launch needs for the n x n system
// (row stride ld): the factor's tiles, the right-hand-side rows and the
// backward-solve products, somewhat more than (ld + 32) x ld.
size_t chol_cluster_ws_doubles(int ld, int n);

// Factorises S (row-major, ld columns, identity padding beyond n, b_schur as
// row ld), solves S x = b and writes x[0..n) -- or sets *solve_ok = 0 and
// leaves x untouched when a pivot is not positive.  S is only read; ws is a
// workspace of chol_cluster_ws_doubles(ld, n) doubles through which the CTAs
// exchange tiles.
cudaError_t chol_cluster_launch(const CholPlan& plan, const double* S, double* ws, int ld, int n, double* x,
                                int* solve_ok, cudaStream_t st);

}  // namespace mcba
