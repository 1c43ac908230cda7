/*
 * g2o_oracle.h -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
 *
 * CPU restatement of the bundle-adjustment path that MCVSLAM runs through
 * g2o (BAoptimizer -> SparseOptimizer -> OptimizationAlgorithmLevenberg ->
 * BlockSolver<6,3> -> LinearSolverEigen).  It exists only to check the CUDA
 * path and to time the reference algorithm on host cores.  Only the test
 * suite, the smoke check and the benchmark's CPU-baseline / reference legs
 * may load it; the product library never links it.
 *
 * Parity status: UNPINNED.  The reference ships no golden vectors or
 * known-answer tests for this path, and its g2o cannot be compiled here
 * (Eigen3, OpenCV, ROS are absent).  The restatement is anchored on the
 * reference's source (file:line citations in g2o_oracle.cpp) and on
 * hand-derived known answers (tests/golden).
 *
 * Problem layout (shared with the product C-ABI bulk loader):
 *   cameras : fx fy cx cy as float (BaseCamera::parameters is
 *             std::vector<float>, modules/camera/BaseCamera.hpp:43),
 *             bf float, T_cam_body as a row-major float 4x4 (cv::Mat CV_32F).
 *   poses   : T_body_world as a row-major float 4x4 (Frame::GetPose()).
 *   points  : world position, float[3] (MapPoint::GetWorldPos()).
 *   edges   : type, pose, point, camera, observation (u, v, u_right) as
 *             float (cv::Point2f / float ru), information scale invSigma2
 *             (float), Huber delta (const float in BAoptimizer.hpp:62-63),
 *             robust flag, level.
 * Vertex order: poses keep their array order, points keep theirs; this
 * equals g2o's id order for problems built the way BAoptimizer builds them
 * (ids handed out in insertion order, src/BAoptimizer.cpp:22-42).
 */
#ifndef MCBA_G2O_ORACLE_H
#define MCBA_G2O_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_EDGE_MONO = 0, ORC_EDGE_STEREO = 1, ORC_EDGE_UNARY = 2 };

typedef struct orc_problem {
  int32_t n_cams;
  const float* cam_K;     /* [n_cams][4] fx fy cx cy */
  const float* cam_bf;    /* [n_cams] */
  const float* cam_Tcb;   /* [n_cams][16] */
  int32_t n_poses;
  const float* pose_Tcw;  /* [n_poses][16] */
  const uint8_t* pose_fixed;
  int32_t n_points;
  const float* point_Xw;  /* [n_points][3] */
  const uint8_t* point_fixed;
  int32_t n_edges;
  const uint8_t* edge_type;
  const int32_t* edge_pose;
  const int32_t* edge_point;
  const int32_t* edge_cam;
  const float* edge_obs;  /* [n_edges][3] */
  const float* edge_info;
  const float* edge_delta;
  const uint8_t* edge_robust;
  const uint8_t* edge_level;
} orc_problem;

typedef struct orc_trial_log {
  int32_t iteration;
  int32_t trial;
  double chi_before;
  double chi_after;
  double lambda;
  double scale;
  double rho;
  int32_t accepted;
  int32_t solve_ok;
} orc_trial_log;

typedef struct orc_result {
  double* pose_qt;        /* [n_poses][7] qx qy qz qw tx ty tz, may be NULL */
  float* pose_Tcw;        /* [n_poses][16], may be NULL */
  double* point_X;        /* [n_points][3], may be NULL */
  double* edge_chi2;      /* [n_edges] chi2 from a final computeError, may be NULL */
  uint8_t* edge_level;    /* [n_edges] levels after filtering, may be NULL */
  orc_trial_log* log;     /* may be NULL */
  int32_t log_cap;
  int32_t n_log;
  int32_t iterations_done;
  int32_t n_active_edges;
  double final_chi2;      /* activeRobustChi2 at the final state */
  double seconds_linearize; /* time in computeActiveErrors-free buildSystem */
  double seconds_total;
  int64_t edges_linearized;
} orc_result;

/* Levenberg-Marquardt over the problem (SparseOptimizer::optimize).
 * n_threads <= 1 runs the serial restatement; > 1 uses OpenMP when built
 * with it.  Returns the g2o return value (iterations, 0 on Fail, -1 when
 * there is nothing to optimise). */
int orc_optimize(const orc_problem* p, int iterations, int n_threads, orc_result* r);

/* PoseEstimation::PoseOptimization restated (src/PoseEstimation.cpp:48-130):
 * `rounds` optimisations of `iters` iterations, chi2 outlier marking with
 * `chi2_thr`, robust kernels dropped after round `drop_robust_round`.
 * Returns nInitialCorrespondences - nBad (0 when fewer than 3 edges). */
int orc_pose_optimization(const orc_problem* p, int rounds, int iters, float chi2_thr,
                          int drop_robust_round, int n_threads, orc_result* r,
                          int* pose_written);

/* PoseEstimation::BoundleAdjustment restated (include/PoseEstimation.hpp:36-119):
 * optimize(n_iter), chi2 >= chi2_thr edges set to level 1, returns the
 * success edge count (always the edge count: the reference never
 * increments nBad) and sets *written when recovery_all would run. */
int orc_local_ba(const orc_problem* p, int iterations, float chi2_thr, int n_threads,
                 orc_result* r, int* written);

/* Per-edge computeError + linearizeOplus at the initial state.
 * err [n][3], J_point [n][3][3] (rows = error dims), J_pose [n][3][6];
 * unused rows (mono edges) are zero. */
int orc_linearize_edges(const orc_problem* p, double* err, double* J_point, double* J_pose);

/* Full (un-reduced) normal equations at the initial state with damping
 * lambda on every diagonal entry: H [(6Kf+3Pf)^2], b [6Kf+3Pf], both in
 * g2o's Hessian index order.  Also the Schur-complement solution x via the
 * BlockSolver path.  Returns the dimension. */
int orc_normal_equations(const orc_problem* p, double lambda, double* H, double* b, double* x_schur,
                         int cap);

/* Flat map tables read by Map::AddKeyFrame's local-BA set-up
 * (src/Map.cpp:140-145): keyframes with their LEFT (0) / WIDE (1)
 * observations, map points with the keyframes bound to them
 * (MapPoint::GetAllKeyFrame), the essential graph, the rig. */
typedef struct orc_map_tables {
  int32_t n_keyframes;
  const int64_t* kf_id;       /* [K] Frame::id */
  const int32_t* obs_begin;   /* [K + 1] */
  const int32_t* obs_point;   /* [O] map point index */
  const uint8_t* obs_object;  /* [O] 0 LEFT, 1 WIDE */
  const float* obs_uv;        /* [O][2] */
  const float* obs_ur;        /* [O] u_right, -1 when none */
  const uint8_t* obs_octave;  /* [O] */
  int32_t n_points;
  const int32_t* mp_kf_begin; /* [P + 1] */
  const int32_t* mp_kf;       /* keyframe indices */
  const int32_t* ess_begin;   /* [K + 1] */
  const int32_t* ess_adj;
  const float* inv_sigma2_left;  /* per octave */
  const float* inv_sigma2_wide;
} orc_map_tables;

/* The local-BA window and its problem in BAoptimizer insertion order. */
typedef struct orc_window_out {
  uint8_t* kf_role;      /* [K] bit 0 optimised, bit 1 anchor (fixed); may be NULL */
  int32_t* pose_kf;      /* [<= K] map keyframe of each problem pose */
  uint8_t* pose_fixed;   /* [<= K] */
  int32_t* point_mp;     /* [<= P] map point of each problem point */
  uint8_t* point_fixed;  /* [<= P] ThisMapPointBeFix */
  int32_t max_edges;
  uint8_t* edge_type;
  int32_t* edge_pose;
  int32_t* edge_point;
  int32_t* edge_cam;     /* 0 LEFT, 1 WIDE */
  float* edge_obs;       /* [E][3] u v u_right (0 for mono edges) */
  float* edge_info;
  float* edge_delta;
  int32_t n_local, n_anchor, n_poses, n_points, n_edges;
} orc_window_out;

/* GrabLocalMap_Mappoint(cur, hop), GrabAnchorKeyFrames, the new keyframe
 * added, then BoundleAdjustment's vertex/edge insertion with
 * ThisMapPointBeFix (window_oracle.cpp).  Returns 0, -1 on bad arguments,
 * -2 when more than max_edges edges. */
int orc_local_window(const orc_map_tables* m, int32_t cur, int32_t hop, orc_window_out* out);

/* Building blocks for known-answer tests. */
void orc_se3_exp(const double update[6], double qt_out[7]);
void orc_mat44f_to_qt(const float T[16], double qt_out[7]);
void orc_qt_to_mat44f(const double qt[7], float T_out[16]);
void orc_huber(double e2, double delta, double rho_out[3]);
void orc_compose(const double a_qt[7], const double b_qt[7], double out_qt[7]);
void orc_map(const double qt[7], const double X[3], double out[3]);

#ifdef __cplusplus
}
#endif
#endif
