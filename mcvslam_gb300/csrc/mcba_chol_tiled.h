// mcba_chol_tiled.h -- blocked FP64 Cholesky solve of reduced camera systems
// larger than the cluster solve takes (mcba_chol_tiled.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace mcba {

// Side stream and events of the lookahead (one set per solver).
struct TiledChol {
  cudaStream_t side = nullptr;
  cudaEvent_t ev_panel = nullptr, ev_rest = nullptr;
};
cudaError_t chol_tiled_setup(TiledChol* t);
void chol_tiled_release(TiledChol* t);

// Row stride of an n x n system for this solve (a multiple of the
// 32-column panel).
int chol_tiled_stride(int n);

// Doubles of workspace the solve needs (diagonal factors, their inverses, the
// backward-substitution partials) for a system of row stride ld.
size_t chol_tiled_ws_doubles(int ld);

// Factorises S in place (row-major, ld columns (chol_tiled_stride(n)), identity padding beyond n,
// b_schur as row ld, which becomes the forward-substituted right-hand side),
// then solves and writes x[0..n) -- unless a pivot is not positive, which sets
// *solve_ok = 0 and leaves x untouched.  Work is issued on st and the side
// stream; when the call returns, st depends on all of it.  The lower
// triangle of S (absent blocks included) is overwritten.
cudaError_t chol_tiled_launch(TiledChol& t, double* S, double* ws, int ld, int n, double* x, int* solve_ok,
                              cudaStream_t st, long long* launches);

}  // namespace mcba
