// mcba_internal.h -- host-side problem model and compiled structure shared by
// the C-ABI layer (mcba_api.cpp) and the device solver (mcba_solver.cu).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include "mcba.h"

namespace mcba {

// SE3 estimate as g2o stores it (types/slam3d/se3quat.h:44-45): unit
// quaternion (x y z w, w >= 0) and translation.
struct QT {
  double q[4];
  double t[3];
};

struct HostCamera {
  float K[4];  // fx fy cx cy
  float bf;
  QT T_cb;     // T_cam_body
};

// std::allocator whose value-initialisation leaves elements uninitialised,
// so resize() on the bulk arrays costs no zero fill (the bulk load writes
// every element right after).
template <typename T>
struct NoInitAlloc : std::allocator<T> {
  template <typename U>
  struct rebind {
    using other = NoInitAlloc<U>;
  };
  NoInitAlloc() = default;
  template <typename U>
  NoInitAlloc(const NoInitAlloc<U>&) {}
  template <typename U>
  void construct(U* p) noexcept {
    ::new (static_cast<void*>(p)) U;
  }
  template <typename U, typename... A>
  void construct(U* p, A&&... a) {
    ::new (static_cast<void*>(p)) U(std::forward<A>(a)...);
  }
};
template <typename T>
using BulkVec = std::vector<T, NoInitAlloc<T>>;

// The graph as the caller built it (vertex and edge ids = insertion order).
struct HostProblem {
  std::vector<HostCamera> cams;
  std::vector<QT> poses;
  std::vector<uint8_t> pose_fixed;
  std::vector<double> points;  // [P][3]
  std::vector<uint8_t> point_fixed;
  std::vector<uint8_t> e_type;
  BulkVec<int32_t> e_pose, e_point, e_cam;
  BulkVec<float> e_obs;  // [E][3]
  BulkVec<float> e_info, e_delta;
  std::vector<uint8_t> e_robust, e_level;
  std::vector<double> u_Xw;  // [U][3] constant points of the unary edges, in edge order

  size_t n_edges() const { return e_type.size(); }
  void clear() {
    cams.clear();
    poses.clear();
    pose_fixed.clear();
    points.clear();
    point_fixed.clear();
    e_type.clear();
    e_pose.clear();
    e_point.clear();
    e_cam.clear();
    e_obs.clear();
    e_info.clear();
    e_delta.clear();
    e_robust.clear();
    e_level.clear();
    u_Xw.clear();
  }
};

// Per-edge record streamed by the linearisation and cost kernels
// (pose-sorted order).  32 bytes.
struct EdgeRec {
  int32_t pose;     // state index of the pose
  int32_t point;    // state index of the point (unary edges: P + unary slot)
  int32_t pose_h;   // free-pose Hessian index or -1
  int32_t point_h;  // free-point Hessian index or -1
  int32_t canon;    // canonical (point-sorted) position, -1 when the point is not free
  uint8_t type, cam, robust, dim;
  float info;
  float delta;
};
static_assert(sizeof(EdgeRec) == 32, "EdgeRec layout");

// Result of initializeOptimization + buildStructure
// (sparse_optimizer.cpp:201-272, block_solver.hpp:103-256), flattened for the
// device: canonical edge order = edges of free points, grouped by point in
// Hessian order and by pose index inside a point.
struct Structure {
  int K = 0, P = 0, U = 0;  // poses, points, unary constant points in state
  int Kf = 0, Lf = 0;       // free poses / free points
  int E = 0;                // active edges
  int Ec = 0;               // active edges with a free point (canonical range)
  std::vector<int32_t> free_pose_ids, free_point_ids;
  std::vector<int32_t> pose_h, point_h;  // id -> Hessian index or -1
  // pose-sorted edge stream
  std::vector<EdgeRec> recs;             // [E]
  std::vector<float> obs;                // [E][3]
  std::vector<int32_t> active_ids;       // [E] original edge id per stream slot
  std::vector<int32_t> chunk_begin;      // [nchunk+1] into recs
  std::vector<int32_t> chunk_pose;       // [nchunk] free pose index or -1
  std::vector<int32_t> pose_chunk_begin; // [Kf+1] chunks of free pose i
  std::vector<int32_t> pose_edge_begin;  // [Kf+1] stream range of free pose i
  // canonical order
  std::vector<int32_t> pt_begin;         // [Lf+1]
  std::vector<int32_t> canon_pose_h;     // [Ec] free pose index or -1
  std::vector<int32_t> canon_point_h;    // [Ec]
  // Schur pairs
  std::vector<int32_t> pair_ij;          // [npairs][2] canonical edge indices
  std::vector<int32_t> pchunk_begin;     // [npchunk+1]
  std::vector<int32_t> pchunk_block;     // [npchunk]
  std::vector<int32_t> block_ab;         // [nblock][2] pose indices a <= b
  std::vector<int32_t> block_chunk_begin;// [nblock+1]
  std::vector<int32_t> pose_canon_list;  // canonical edges of free pose i (for b_schur), CSR
  std::vector<int32_t> pose_canon_begin; // [Kf+1]
};

// Compiles the active structure; returns false when there is nothing to optimise.
bool compile_structure(const HostProblem& hp, Structure& s);

// Growable device buffer (reused across calls; never shrinks).
template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t n) {
    if (n <= cap && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    const size_t want = std::max<size_t>(n, 1);
    cudaError_t e = cudaMalloc(&p, want * sizeof(T));
    if (e == cudaSuccess) cap = want;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
};

// Structure compilation on the device (mcba_compile.cu): the same arrays as
// compile_structure, built from the raw edge list by scans, a per-point
// ordering and stable multi-way partitions.
struct StructureSizes {
  int K, P, U, Kf, Lf, E, Ec, nchunk, npairs, nblk, npc;
};
struct DeviceStructureOut {
  EdgeRec* recs;
  float* obs;              // [E][3]
  int* chunk_begin;        // [nchunk+1]
  int* chunk_pose;         // [nchunk]
  int* pose_chunk_begin;   // [Kf+1]
  int* pt_begin;           // [Lf+1]
  int* canon_pose_h;       // [Ec]
  int* canon_point_h;      // [Ec]
  int2* pairs;             // [npairs]
  int* pchunk_begin;       // [npc+1]
  int* block_ab;           // [nblk][2]
  int* block_chunk_begin;  // [nblk+1]
  int* pose_canon_begin;   // [Kf+1]
  int* pose_canon_list;    // [pose_canon_begin[Kf]]
  int* free_pose_ids;      // [Kf]
  int* free_point_ids;     // [Lf]
};
class DeviceCompiler;
DeviceCompiler* compiler_create();
void compiler_destroy(DeviceCompiler* c);
// Uploads the raw graph and computes every size (one device-to-host read).
int compiler_phase1(DeviceCompiler* c, const HostProblem& hp, cudaStream_t st, StructureSizes* sz, int64_t* h2d,
                    std::string* err);
// Fills the caller's buffers (sized from phase 1).
int compiler_phase2(DeviceCompiler* c, const DeviceStructureOut& out, cudaStream_t st, std::string* err);

// Device solver (mcba_solver.cu).
class Solver;
Solver* solver_create(int device, int precision, void* stream, std::string* err);
void solver_destroy(Solver* s);
// Frees the idle solvers kept for reuse (device < 0: all devices); returns how many.
int solver_release_cached(int device);

struct SolveResult {
  int status = MCBA_OK;
  int iterations = 0;
  int trials = 0;
  double initial_chi2 = 0, final_chi2 = 0, lambda = 0;
  double ms_total = 0, ms_linearize = 0;
  double ms_phase[MCBA_NUM_PHASES] = {0};
  int n_phase[MCBA_NUM_PHASES] = {0};
  int64_t launches = 0, h2d = 0, d2h = 0;
  std::vector<mcba_trial_log> log;
  std::vector<double> hpp;  // [Kf][36] of the last linearisation (for dump)
};

struct RunOptions {
  int iterations = 10;
  double tau = 1e-5;
  int max_trials = 10;
  bool use_graph = true;
  bool profile = false;
};

// Uploads state and structure (keeps a device copy of the initial state).
// With st == nullptr the structure is compiled on the device; the sizes of
// the compiled structure are returned in *sizes either way.  Returns
// MCBA_ERR_EMPTY when nothing is left to optimise.
int solver_upload(Solver* s, const HostProblem& hp, const Structure* st, StructureSizes* sizes, SolveResult& out,
                  std::string* err);
// Runs LM on the uploaded problem; restore = start again from the uploaded
// initial state.
int solver_run(Solver* s, const RunOptions& o, bool restore, SolveResult& out, std::string* err);
// LM on several uploaded problems at once: every solver's solve (restored
// from its uploaded initial state) is a branch of one CUDA graph, launched
// once.  ms_device: event time of that launch.
int solver_run_batch(Solver* const* ss, int n, const RunOptions& o, SolveResult* outs, double* ms_device,
                     std::string* err);
// The same batch in one persistent launch: clusters of CTAs take the
// windows from a device work queue and each runs a window's whole LM solve
// (k_windows); the cluster size is chosen by timing the batch on its first
// call.  Every problem must share the device and the precision, with at
// most 384 reduced unknowns.  cluster_ctas (may be null): in, 0 to let the
// autotuner choose or 4, 8, 16 to use that size; out, the size used.
int solver_run_batch_persistent(Solver* const* ss, int n, const RunOptions& o, SolveResult* outs, double* ms_device,
                                int* cluster_ctas, std::string* err);
// Copies the current device state into hp.
int solver_download(Solver* s, HostProblem& hp, SolveResult& out, std::string* err);
bool solver_has_upload(const Solver* s);

// chi2 of every edge at the current state (FP64), device computed.
int solver_edge_chi2(Solver* s, const HostProblem& hp, std::vector<double>& chi2, std::string* err);

}  // namespace mcba
