/*
 * mcba.h -- C ABI of the GB300 bundle-adjustment solver (libmcba.so).
 *
 * Drop-in replacement for MCVSLAM's BAoptimizer (include/BAoptimizer.hpp:29-80,
 * src/BAoptimizer.cpp:13-143 of the reference) and for the two PoseEstimation
 * drivers built on it (include/PoseEstimation.hpp:35-119,
 * src/PoseEstimation.cpp:48-151).  Every entry point takes plain pointers and
 * sizes, returns an int status (MCBA_OK == 0) and never throws.  A problem
 * handle is used by one host thread at a time; distinct handles are
 * independent.  All numeric inputs cross the boundary in the precision the
 * reference hands to g2o (float poses, points, pixels, information and Huber
 * thresholds) and the solver keeps its state in FP64 internally.
 */
#ifndef MCBA_H
#define MCBA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MCBA_ABI_VERSION 1

/* ------------------------------------------------------------ status -- */
enum {
  MCBA_OK = 0,
  MCBA_ERR_INVALID = 1,     /* bad argument: unknown id, NULL pointer, bad size */
  MCBA_ERR_EMPTY = 2,       /* nothing to optimise (g2o: "0 vertices to optimize") */
  MCBA_ERR_NOT_PD = 3,      /* reduced camera system not positive definite */
  MCBA_ERR_NONFINITE = 4,   /* NaN/Inf in the inputs */
  MCBA_ERR_TIMEOUT = 5,     /* a bounded device wait gave up */
  MCBA_ERR_CUDA = 6,        /* CUDA runtime error (see mcba_last_error) */
  MCBA_ERR_NOMEM = 7,       /* device or host allocation failed */
  MCBA_ERR_NO_DEVICE = 8,   /* no CUDA device */
  MCBA_ERR_TOO_LARGE = 9    /* request above a documented maximum */
};

/* Edge kinds of include/OptimizeTypes.hpp */
enum {
  MCBA_EDGE_MONO = 0,   /* EdgeSE3XYZ2Camera: point -> body pose through T_cam_body (hpp:70-117) */
  MCBA_EDGE_STEREO = 1, /* EdgeStereoSE3ProjectXYZ: (u, v, u_right), pose used as T_cam_world (hpp:119-157) */
  MCBA_EDGE_UNARY = 2   /* EdgeSE3XYZ2CameraOnlyPose: constant world point (hpp:20-68) */
};

enum {
  MCBA_PREC_FP64 = 0,  /* plain: every step in FP64 (matches g2o) */
  MCBA_PREC_MIXED = 1  /* FP32 residuals/Jacobians/Schur blocks, FP64 Cholesky, LM test and retraction */
};

typedef struct mcba_problem mcba_problem;

typedef struct mcba_options {
  int32_t precision;   /* MCBA_PREC_* */
  int32_t device;      /* CUDA device ordinal */
  double tau;          /* LM initial damping factor, g2o default 1e-5 (optimization_algorithm_levenberg.cpp:43) */
  int32_t max_trials;  /* maxTrialsAfterFailure, default 10 (optimization_algorithm_levenberg.cpp:50) */
  int32_t use_graph;   /* 1: run the LM loop as one CUDA graph with device-side control */
  int32_t profile;     /* 1: time every phase with CUDA events (mcba_stats.ms_phase) */
  void* stream;        /* cudaStream_t to run on, NULL for a library-owned stream */
  int32_t host_structure; /* 1: compile the problem structure on the host (default 0: on the device) */
} mcba_options;

/* Phases timed when mcba_options.profile is set, named after g2o's
 * G2OBatchStatistics fields (core/batch_stats.h:40-76). */
enum {
  MCBA_PHASE_LINEARIZE = 0,   /* timeQuadraticForm: per-edge residual/Jacobian/quadratic terms */
  MCBA_PHASE_REDUCE = 1,      /* Hpp / Hll / b segmented sums (+ lambda init) */
  MCBA_PHASE_SCHUR_EDGE = 2,  /* timeSchurComplement: Y = Hpl Dinv per edge */
  MCBA_PHASE_SCHUR_PAIRS = 3, /* timeSchurComplement: reduced-camera block products */
  MCBA_PHASE_SCHUR_ASSEMBLE = 4, /* dense reduced camera matrix + b_schur */
  MCBA_PHASE_CHOLESKY = 5,    /* timeLinearSolver: FP64 factorisation and solves */
  MCBA_PHASE_UPDATE = 6,      /* timeUpdate: back-substitution, retraction */
  MCBA_PHASE_COST = 7,        /* timeResiduals: activeRobustChi2 + LM decision */
  MCBA_NUM_PHASES = 8
};

typedef struct mcba_stats {
  int32_t iterations;        /* g2o optimize() return value */
  int32_t trials;            /* LM trials run (linear solves) */
  int32_t n_active_edges;
  int32_t n_free_poses;
  int32_t n_free_points;
  int32_t status;            /* MCBA_* of the last solve */
  double initial_chi2;       /* activeRobustChi2 before the first iteration */
  double final_chi2;         /* activeRobustChi2 at the returned state */
  double lambda;             /* damping after the last trial */
  int64_t edges_linearized;  /* active edges x iterations */
  double ms_total;           /* device time of the whole solve (CUDA events) */
  double ms_linearize;       /* device time of the linearisation phases */
  double ms_host_prepare;    /* host time of structure compilation and upload */
  double ms_phase[MCBA_NUM_PHASES];   /* device time per phase (profile option) */
  int32_t n_phase[MCBA_NUM_PHASES];   /* timed launches per phase */
  int64_t kernel_launches;   /* device kernels launched by the solve */
  int64_t h2d_bytes;         /* host-to-device bytes copied by the call */
  int64_t d2h_bytes;         /* device-to-host bytes copied by the call */
} mcba_stats;

typedef struct mcba_trial_log {
  int32_t iteration;
  int32_t trial;
  double chi_before;
  double chi_after;
  double lambda;
  double scale;
  double rho;
  int32_t accepted;
  int32_t solve_ok;
} mcba_trial_log;

/* ------------------------------------------------------- life cycle -- */
int mcba_abi_version(void);
const char* mcba_status_string(int status);
void mcba_default_options(mcba_options* opt);
/* Handles destroyed with a library-owned stream leave their device workspace
 * (buffers, pinned staging, stream, captured graph) in a small per-device
 * cache that the next mcba_create on that device and precision reuses.  This
 * frees the cached workspaces of one device (device < 0: of every device).
 * No reference counterpart: g2o allocates per optimizer. */
int mcba_release_cached(int32_t device);
int mcba_device_count(int* count);

/* Replaces BAoptimizer::BAoptimizer (src/BAoptimizer.cpp:13-18). */
int mcba_create(const mcba_options* opt, mcba_problem** out);
/* Replaces BAoptimizer::~BAoptimizer; frees every host and device buffer. */
int mcba_destroy(mcba_problem* p);
/* Message of the last error on this handle ("" when none). */
const char* mcba_last_error(const mcba_problem* p);
/* Drops every vertex and edge, keeps the options and device buffers. */
int mcba_clear(mcba_problem* p);

/* ------------------------------------------------------- graph build -- */
/* Camera model Pinhole (modules/camera/Pinhole.cpp:55-60,105-116): K = fx fy cx
 * cy, bf for stereo edges, T_cam_body row-major float 4x4 (the Tcb argument of
 * EdgeSE3XYZ2Camera, include/OptimizeTypes.hpp:74, converted as
 * Converter::toSE3Quat, src/Converter.cc:31-39). */
int mcba_add_camera(mcba_problem* p, const float K[4], float bf, const float T_cam_body[16], int32_t* id);

/* BAoptimizer::addKeyFrame (src/BAoptimizer.cpp:22-31): T_body_world as a
 * row-major float 4x4; fixed as in setFixed.  (The reference also fixes the
 * keyframe with id 0; callers pass that as fixed.) */
int mcba_add_keyframe(mcba_problem* p, const float T_body_world[16], int fixed, int32_t* id);
/* Same with the estimate given as FP64 quaternion (x y z w) + translation. */
int mcba_add_keyframe_qt(mcba_problem* p, const double qt[7], int fixed, int32_t* id);

/* BAoptimizer::addMapppint (src/BAoptimizer.cpp:33-42): marginalised point. */
int mcba_add_mappoint(mcba_problem* p, const float Xw[3], int fixed, int32_t* id);

/* BAoptimizer::addEdge / addEdgeToBody (src/BAoptimizer.cpp:45-65,90-108):
 * EdgeSE3XYZ2Camera with the camera's T_cam_body, information
 * inv_sigma2 * I, Huber kernel of threshold huber_delta (<= 0: no kernel). */
int mcba_add_edge_mono(mcba_problem* p, int32_t keyframe, int32_t mappoint, int32_t camera, float u,
                       float v, float inv_sigma2, float huber_delta, int32_t* id);
/* BAoptimizer::addEdgeStereo (src/BAoptimizer.cpp:67-88). */
int mcba_add_edge_stereo(mcba_problem* p, int32_t keyframe, int32_t mappoint, int32_t camera, float u,
                         float v, float u_right, float inv_sigma2, float huber_delta, int32_t* id);
/* EdgeSE3XYZ2CameraOnlyPose (include/OptimizeTypes.hpp:20-68): unary edge on a
 * keyframe with a constant world point. */
int mcba_add_edge_posonly(mcba_problem* p, int32_t keyframe, int32_t camera, const float Xw[3], float u,
                          float v, float inv_sigma2, float huber_delta, int32_t* id);

/* Bulk form of the three edge calls: type[n] (MCBA_EDGE_*), obs[n][3]
 * (u, v, u_right), Xw[n][3] only read for unary edges (may be NULL when there
 * are none).  Ids are consecutive from *first_id. */
int mcba_add_edges(mcba_problem* p, int32_t n, const uint8_t* type, const int32_t* keyframe,
                   const int32_t* mappoint, const int32_t* camera, const float* obs, const float* Xw,
                   const float* inv_sigma2, const float* huber_delta, int32_t* first_id);

/* Whole-problem bulk loader in the layout of the synthetic generator:
 * cameras, keyframes (float 4x4), points, edges (unary edges take their
 * constant point from point_Xw[edge_point]).  Equivalent to the add_* calls
 * in array order. */
typedef struct mcba_problem_desc {
  int32_t n_cams;
  const float* cam_K;     /* [n_cams][4] */
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
  const uint8_t* edge_robust; /* may be NULL: all robust */
  const uint8_t* edge_level;  /* may be NULL: all level 0 */
} mcba_problem_desc;
int mcba_load(mcba_problem* p, const mcba_problem_desc* d);

/* BAoptimizer::getEdgeSize (include/BAoptimizer.hpp:43). */
int mcba_edge_count(const mcba_problem* p, int32_t* n);
int mcba_vertex_count(const mcba_problem* p, int32_t* n_keyframes, int32_t* n_mappoints);

/* ------------------------------------------------------------ solve -- */
/* BAoptimizer::optimize(n) (src/BAoptimizer.cpp:110-114): initializeOptimization
 * on level-0 edges, then n Levenberg-Marquardt iterations with g2o's damping
 * rules.  stats may be NULL. */
int mcba_optimize(mcba_problem* p, int32_t iterations, mcba_stats* stats);

/* Device-resident re-solve, for timing with the inputs already in device
 * memory: mcba_prepare compiles and uploads the problem once (and keeps a
 * device copy of the initial estimates); every mcba_solve_prepared restores
 * that initial state on the device and runs the LM iterations without any
 * host<->device copy of problem data.  The result stays on the device until
 * mcba_fetch_state copies it back into the handle (mcba_get_* then read it). */
int mcba_prepare(mcba_problem* p);
int mcba_solve_prepared(mcba_problem* p, int32_t iterations, mcba_stats* stats);
int mcba_fetch_state(mcba_problem* p);

/* Per-trial record of the last optimize (iteration, trial, chi2 before/after,
 * lambda, scale, rho, accepted, solve_ok). */
int mcba_trial_log_get(const mcba_problem* p, mcba_trial_log* out, int32_t cap, int32_t* n);

/* ----------------------------------------------------- edge control -- */
/* e->computeError(); e->chi2() for every edge at the current estimate (the
 * input of the filter callbacks, src/PoseEstimation.cpp:98-116,132-151). */
int mcba_edge_chi2(mcba_problem* p, double* chi2);
/* e->setLevel / e->level(): 0 = optimised, 1 = excluded. */
int mcba_set_edge_levels(mcba_problem* p, const uint8_t* levels);
int mcba_get_edge_levels(const mcba_problem* p, uint8_t* levels);
/* e->setRobustKernel(0) when robust[i] == 0, restores the Huber kernel otherwise. */
int mcba_set_edge_robust(mcba_problem* p, const uint8_t* robust);

/* ---------------------------------------------------------- read back -- */
/* BAoptimizer::eval(KeyFrame) (src/BAoptimizer.cpp:121-126): float 4x4
 * T_body_world as Converter::toCvMat (src/Converter.cc:41-52). */
int mcba_get_keyframe(const mcba_problem* p, int32_t id, float T_body_world[16]);
int mcba_get_keyframe_qt(const mcba_problem* p, int32_t id, double qt[7]);
/* BAoptimizer::eval(MapPointRef) (src/BAoptimizer.cpp:128-132). */
int mcba_get_mappoint(const mcba_problem* p, int32_t id, float Xw[3]);
/* Bulk FP64 state: qt[n_keyframes][7], X[n_mappoints][3] (either may be NULL). */
int mcba_get_state(const mcba_problem* p, double* qt, double* X);
/* Overwrites the FP64 estimates (warm start; quaternions are renormalised
 * with w >= 0 as SE3Quat does).  Either pointer may be NULL. */
int mcba_set_state(mcba_problem* p, const double* qt, const double* X);

/* BAoptimizer::DumpCalculationGraph (src/BAoptimizer.cpp:116-119): writes the
 * pose Hessian Hpp of the last linearisation as upper-triangular Octave text. */
int mcba_dump_hessian(mcba_problem* p, const char* path);

/* ------------------------------------------------------------ drivers -- */
/* PoseEstimation::PoseOptimization (src/PoseEstimation.cpp:48-130) on a
 * problem holding one free keyframe and fixed points: `rounds` optimisations
 * of `iterations` each, edges with chi2 >= chi2_threshold set to level 1 after
 * each round, robust kernels dropped after round `drop_robust_round`, early
 * stop when fewer than 10 edges remain.  *inliers = nInitial - nBad (0 with
 * fewer than 3 edges); *pose_written = whether the reference would call
 * SetPose.  Edge levels are left as the filter set them. */
int mcba_pose_optimization(mcba_problem* p, int32_t rounds, int32_t iterations, float chi2_threshold,
                           int32_t drop_robust_round, int32_t* inliers, int32_t* pose_written);

/* PoseEstimation::BoundleAdjustment (include/PoseEstimation.hpp:36-119):
 * optimize(iterations), then FilterCallBack_Chi2 on every level-0 edge
 * (chi2 >= chi2_threshold -> level 1).  *success_edges reproduces the
 * reference's return value (the edge count: nBad is never incremented there);
 * *written = whether recovery_all would run (success_edges > 10). */
int mcba_local_ba(mcba_problem* p, int32_t iterations, float chi2_threshold, int32_t* success_edges,
                  int32_t* written);

/* ------------------------------------------- local-BA window of a map -- */
/* Flat tables of a SLAM map, as Map::AddKeyFrame reads them before its local
 * BA (src/Map.cpp:140-145): keyframes with the map points their LEFT (0) and
 * WIDE (1) objects observe, map points with the keyframes bound to them
 * (MapPoint::GetAllKeyFrame), the essential graph, and the rig.  Host arrays.
 * Each (keyframe, object, map point) appears at most once, as in an Object.
 * Frame ids must lie in [0, 2^39) and n_keyframes below 2^24. */
typedef struct mcba_map_desc {
  int32_t n_keyframes;
  const int64_t* kf_id;        /* [K] Frame::id */
  const float* kf_Tcw;         /* [K][16] T_body_world, row-major (Frame::GetPose) */
  const int32_t* obs_begin;    /* [K + 1] observations of each keyframe */
  const int32_t* obs_point;    /* [O] map point */
  const uint8_t* obs_object;   /* [O] 0 LEFT, 1 WIDE */
  const float* obs_uv;         /* [O][2] keypoint position */
  const float* obs_ur;         /* [O] u_right of a LEFT keypoint, -1 when none */
  const uint8_t* obs_octave;   /* [O] keypoint octave */
  int32_t n_points;
  const float* mp_Xw;          /* [P][3] MapPoint::GetWorldPos */
  const int32_t* mp_kf_begin;  /* [P + 1] keyframes bound to each map point */
  const int32_t* mp_kf;
  const int32_t* ess_begin;    /* [K + 1] essential-graph neighbours */
  const int32_t* ess_adj;
  int32_t n_levels;
  const float* inv_sigma2_left;  /* [n_levels] mvInvLevelSigma2 of the left extractor */
  const float* inv_sigma2_wide;  /* [n_levels] of the wide extractor */
  float K_left[4];             /* fx fy cx cy of the LEFT camera (T_cam_body = I) */
  float K_wide[4];             /* of the WIDE camera */
  float T_wide_body[16];       /* T_cam_body of the WIDE camera (kf->Twl) */
  float bf;                    /* stereo baseline x fx (kf->bf) */
} mcba_map_desc;

typedef struct mcba_window_info {
  int32_t n_local;         /* keyframes optimised, the new one included */
  int32_t n_anchor;        /* fixed anchor keyframes */
  int32_t n_poses, n_points, n_fixed_points, n_edges;
} mcba_window_info;

/* The local BA set-up of Map::AddKeyFrame for keyframe `cur` on the GPU
 * (src/Map.cpp:142-145): GrabLocalMap_Mappoint(cur, hop) (src/Map.cpp:730-756),
 * GrabAnchorKeyFrames (src/Map.cpp:775-796), cur added, then the vertex and
 * edge insertion of PoseEstimation::BoundleAdjustment
 * (include/PoseEstimation.hpp:36-97) with ThisMapPointBeFix per map point
 * (src/PoseEstimation.cpp:153-163) -- replacing its hash-set walks and per-edge
 * allocations.  The problem is loaded into p (camera 0 LEFT, camera 1 WIDE):
 * poses are the anchors then the window keyframes in ascending map index,
 * points in order of first edge, edges in the insertion loop's order (each
 * keyframe's LEFT observations, then its WIDE ones, in table order).  Then
 * mcba_local_ba(p, 10, 5.991, ...) is BoundleAdjustment's optimise and
 * filter.  Outputs (each may be NULL): kf_role [K] (bit 0 optimised, bit 1
 * anchor), pose_kf [<= K] map keyframe of each pose, point_mp [<= P] map
 * point of each point, point_fixed [<= P] ThisMapPointBeFix.
 * Errors: MCBA_ERR_INVALID for bad arguments or tables (an index or CSR range
 * out of bounds). */
int mcba_local_window(mcba_problem* p, const mcba_map_desc* map, int32_t cur, int32_t hop, uint8_t* kf_role,
                      int32_t* pose_kf, int32_t* point_mp, uint8_t* point_fixed, mcba_window_info* info);

/* ---------------------------------------------- Hamming k = 2 matching -- */
/* Matcher::KnnMatch over descriptor lists (src/Matcher.cpp:245-302): for
 * each of nq 32-byte query descriptors, the best and second-best of nt train
 * descriptors by Hamming distance (HammingDistance, include/Matcher.hpp:19-31),
 * ties to the smaller train index, unfilled slots (999, 0) as the reference
 * initialises them.  idx and dist receive [nq][2].  keep (may be NULL)
 * receives FilterRatio(ratio) && FilterThreshold(max_dist) per query, the
 * filters the callers apply (src/Matcher.cpp:23-34,100-111; the reference's
 * defaults are 0.6 and 46).
 * mcba_knn_hamming_device: device pointers (query and train 16-byte
 * aligned), on `stream`; its chunk scratch is cached per device, so calls that
 * may overlap on one device must be serialised by the caller.
 * mcba_knn_hamming: host buffers, copies in and out inside the call;
 * *ms_device (may be NULL) receives the kernel time. */
int mcba_knn_hamming_device(const uint8_t* query, int32_t nq, const uint8_t* train, int32_t nt, int32_t* idx,
                            int32_t* dist, float ratio, int32_t max_dist, uint8_t* keep, void* stream);
int mcba_knn_hamming(int32_t device, const uint8_t* query, int32_t nq, const uint8_t* train, int32_t nt,
                     int32_t* idx, int32_t* dist, float ratio, int32_t max_dist, uint8_t* keep, double* ms_device);

/* ------------------------------- map-point projection + windowed match -- */
/* Object::ProjectBunchMapPoints (src/Object.cpp:208-236) for a batch of
 * objects (one camera of one frame each; Tracker.cpp:90-91,128-129 make two
 * such calls per frame).  For every map point of an object, in visit order:
 * project with the object's pose and pinhole camera (R * X + t, then
 * Pinhole::project, modules/camera/Pinhole.cpp:45-47), gather the keypoints
 * of the 30 x 30 grid within r_threshold * mvScaleFactor[level] of the
 * projection (GetFeaturesInArea, src/Object.cpp:263-300), k = 2 Hamming match
 * of the map point's descriptor against them, FilterRatio(ratio) and
 * FilterThreshold(max_dist) (src/Object.cpp:226; the reference passes the
 * defaults 0.6 and 46), and bind the best keypoint (AddMapPoint,
 * src/Object.cpp:113-137). */
typedef struct mcba_projection_batch {
  int32_t n_objects;
  const float* obj_Rt;       /* [n_objects][12] camera from world: R row-major, then t */
  const float* obj_K;        /* [n_objects][4] fx fy cx cy */
  const int32_t* obj_size;   /* [n_objects][2] image cols, rows */
  const float* obj_radius;   /* [n_objects] r_threshold */
  const float* obj_scale;    /* [n_objects][n_levels] mvScaleFactor of the object's extractor */
  int32_t n_levels;
  float ratio;               /* FilterRatio */
  int32_t max_dist;          /* FilterThreshold */
  const int32_t* kp_begin;   /* [n_objects + 1] keypoint ranges, kp_begin[0] = 0 */
  const float* kp_xy;        /* [n_kp][2] keypoint pixel position */
  const uint8_t* kp_desc;    /* [n_kp][32] keypoint descriptors */
  const int32_t* mp_begin;   /* [n_objects + 1] map-point ranges, in visit order, mp_begin[0] = 0 */
  const float* mp_X;         /* [n_mp][3] world position */
  const uint8_t* mp_desc;    /* [n_mp][32] MapPoint::GetDesp */
  const int32_t* mp_level;   /* [n_mp] MapPoint::level, in [0, n_levels) */
  const int32_t* mp_id;      /* [n_mp] the caller's handle, written into kp_bind */
  const int32_t* mp_prev_kp; /* [n_mp] object-local keypoint the map point is bound to before the call
                                (Object::mMP2IDX), or -1; NULL = none bound */
} mcba_projection_batch;

/* Host buffers.  kp_bind [n_kp] (in/out) holds each keypoint's bound map-point
 * handle or -1 (Object::mIDX2MP) and is updated as the reference's sequence of
 * AddMapPoint calls leaves it; mp_match [n_mp] receives the object-local
 * keypoint each map point matched or -1 (its ProjectResRecord flag);
 * obj_count [n_objects] the returned counts.  *ms_device (may be NULL): kernel
 * time.  Invalid levels, ranges or non-finite inputs are errors. */
int mcba_project_match(int32_t device, const mcba_projection_batch* batch, int32_t* kp_bind, int32_t* mp_match,
                       int32_t* obj_count, double* ms_device);
/* The same with every pointer in *batch and the outputs in device memory
 * (kp_desc and mp_desc 16-byte aligned, kp_xy 8-byte aligned), on `stream`;
 * n_kp = kp_begin[n_objects], n_mp = mp_begin[n_objects].  The contents are
 * not validated (out-of-range levels or keypoints give no match); the grid
 * scratch is cached per device, so overlapping calls on one device must be
 * serialised by the caller. */
int mcba_project_match_device(const mcba_projection_batch* batch, int32_t n_kp, int32_t n_mp, int32_t* kp_bind,
                              int32_t* mp_match, int32_t* obj_count, void* stream);

/* ------------------------------------------------------ stereo matching -- */
/* Frame::ComputeStereoMatch (src/Frame.cpp:150-325) for a batch of rectified
 * stereo frames: for each left keypoint, the right keypoints whose row band
 * (10 x mvScaleFactor[octave] rows around their y) covers its row, within one
 * octave and inside the disparity range [1, min(bf / b, 1000)]; k = 2 Hamming
 * match with FilterRatio(0.70) and FilterThreshold(34); 11 x 11 SAD of
 * centre-subtracted patches at the keypoint's pyramid level over 11 offsets;
 * parabola sub-pixel fit; and the per-frame median filter of the best SADs.
 * The pyramid tables are the left extractor's, as in the reference. */
#define MCBA_MAX_LEVELS 32
typedef struct mcba_stereo_batch {
  int32_t n_frames;
  int32_t n_levels;                      /* <= MCBA_MAX_LEVELS */
  float scale[MCBA_MAX_LEVELS];          /* mvScaleFactor */
  float inv_scale[MCBA_MAX_LEVELS];      /* mvInvScaleFactor */
  int32_t level_rows[MCBA_MAX_LEVELS];   /* mvImagePyramid[l].rows (left and right alike) */
  int32_t level_cols[MCBA_MAX_LEVELS];   /* mvImagePyramid[l].cols */
  int64_t level_offset[MCBA_MAX_LEVELS]; /* byte offset of level l in one image's pyramid, rows packed */
  int64_t pyr_bytes;                     /* bytes of one image's pyramid */
  int32_t image_rows;                    /* left image height: rows of the row table (<= 8192) */
  float b;                               /* baseline (minZ) */
  float bf;                              /* baseline x fx */
  const uint8_t* left_pyr;               /* [n_frames][pyr_bytes] */
  const uint8_t* right_pyr;              /* [n_frames][pyr_bytes] */
  const int32_t* left_begin;             /* [n_frames + 1], left_begin[0] = 0 */
  const float* left_xy;                  /* [n_left][2] */
  const int32_t* left_oct;               /* [n_left] octave */
  const uint8_t* left_desc;              /* [n_left][32] */
  const int32_t* right_begin;            /* [n_frames + 1], right_begin[0] = 0 */
  const float* right_xy;                 /* [n_right][2] */
  const int32_t* right_oct;              /* [n_right] */
  const uint8_t* right_desc;             /* [n_right][32] */
} mcba_stereo_batch;

/* Host buffers: u_right and depth [n_left] receive the right-image u and
 * bf / disparity of each left keypoint, -1 where there is none (Frame::u_right,
 * Frame::depth_left).  Invalid octaves or tables, non-finite keypoints are
 * errors.  Where the reference reads outside its arrays the result is
 * defined: band rows outside the image are dropped, a right window starting
 * left of column 0 gives no match, a frame without matches skips the median
 * filter. */
int mcba_stereo_match(int32_t device, const mcba_stereo_batch* batch, float* u_right, float* depth,
                      double* ms_device);
/* The same with the batch's pointers and the outputs in device memory
 * (descriptors 16-byte aligned, positions 8-byte aligned; the tables in the
 * struct stay host values), on `stream`; n_left = left_begin[n_frames],
 * n_right = right_begin[n_frames].  Contents are not validated; the scratch is
 * cached per device, so overlapping calls on one device must be serialised. */
int mcba_stereo_match_device(const mcba_stereo_batch* batch, int32_t n_left, int32_t n_right, float* u_right,
                             float* depth, void* stream);

/* ------------------------------------------- batched local-BA windows -- */
/* Many independent local-BA windows solved together (the windows of config
 * 4): PoseEstimation::BoundleAdjustment (include/PoseEstimation.hpp:36-119)
 * on each window, with the n LM loops as independent branches of one CUDA
 * graph launched once (no host round trip between windows or trials).
 * mcba_batch_prepare compiles and uploads every handle's problem (as
 * mcba_prepare); mcba_batch_solve restores each uploaded initial state and
 * runs `iterations` LM iterations on all of them; mcba_fetch_state then
 * reads one window's estimates back.  All handles must be on one device; the
 * LM options (tau, max_trials) of problems[0] apply to the batch.  stats may
 * be NULL, else it receives n entries; ms_device (may be NULL) the device
 * time of the launch. */
int mcba_batch_prepare(mcba_problem* const* problems, int32_t n);
int mcba_batch_solve(mcba_problem* const* problems, int32_t n, int32_t iterations, mcba_stats* stats,
                     double* ms_device);
/* The same windows (prepared by mcba_batch_prepare) in ONE persistent kernel
 * launch: thread-block clusters stay resident and take windows from a device
 * work queue, largest first, each cluster running one window's whole LM
 * solve (BoundleAdjustment's optimize, include/PoseEstimation.hpp:102-105,
 * with g2o's LM of optimization_algorithm_levenberg.cpp:56-143) with the
 * same arithmetic in the same order as mcba_optimize, so every window's
 * trial log, cost and estimates equal its single solve's.  The number of
 * CTAs per window (the cluster size: 4, 8 or 16) is chosen on the first
 * call for a batch by timing each candidate, unless *cluster_ctas is 4, 8 or
 * 16 on entry (then that size is used); NULL or 0 asks for the autotuner,
 * and *cluster_ctas (when not NULL) receives the size used.  All handles must share the device and the precision, and
 * each window's reduced camera system must have at most 384 unknowns (64
 * free keyframes); MCBA_ERR_INVALID otherwise. */
int mcba_batch_solve_persistent(mcba_problem* const* problems, int32_t n, int32_t iterations, mcba_stats* stats,
                                double* ms_device, int32_t* cluster_ctas);

/* --------------------------------------------- batched pose-only solve -- */
/* Many independent PoseEstimation::PoseOptimization problems
 * (src/PoseEstimation.cpp:48-130) of uneven size in one device pass: a
 * persistent kernel takes problems from a work queue, one CTA per problem,
 * and runs `rounds` x `iterations` of g2o's LM on the problem's 6-dof body
 * pose with the reference's outlier rules (chi2 >= chi2_threshold -> level 1,
 * robust kernels dropped after round drop_robust_round, early stop below 10
 * edges).  Problem i owns the unary edges [edge_begin[i], edge_begin[i+1]).
 *   poses_qt   [n][7]   in: T_body_world (x y z w tx ty tz); out: the result
 *                       when the reference would call SetPose, else unchanged
 *   edge_cam [E], edge_obs [E][2], edge_Xw [E][3], edge_info [E], edge_delta [E]
 *   edge_level [E]      out: 1 for edges classified as outliers
 *   inliers    [n]      out: nInitial - nBad (0 with fewer than 3 edges)
 *   ms_device           out: device time of the batch (may be NULL)
 * cam_K [C][4] and cam_Tcb [C][16] describe the rig shared by all problems.
 * The launch configuration (threads per CTA, CTAs per SM) is chosen by a
 * small autotuner on the first call for each batch shape. */
int mcba_batch_pose_only(int32_t device, int32_t precision, int32_t n, const int32_t* edge_begin,
                         int32_t n_cams, const float* cam_K, const float* cam_Tcb, const int32_t* edge_cam,
                         const float* edge_obs, const float* edge_Xw, const float* edge_info,
                         const float* edge_delta, int32_t rounds, int32_t iterations, float chi2_threshold,
                         int32_t drop_robust_round, double* poses_qt, uint8_t* edge_level, int32_t* inliers,
                         double* ms_device);

/* -------------------------------------------- reprojection primitives -- */
/* Device-pointer entry points behind the autograd harness (no host copies;
 * all pointers are device memory, stream is a cudaStream_t or NULL).  They
 * expose EdgeSE3XYZ2Camera's computeError / linearizeOplus
 * (include/OptimizeTypes.hpp:80-113) plus the rig-extrinsic Jacobian.
 * Forward: residual r = obs - pi(T_cb * T_bw * X) of n mono edges, with
 *   pose_qt [n][7] (T_body_world), ext_qt [n][7] (T_cam_body), X [n][3],
 *   K [n][4], obs [n][2]  ->  res [n][2].  pose_delta / ext_delta [n][6]
 *   (may be NULL) are applied first as T <- exp(delta) * T.
 * Backward: given grad_res [n][2], writes the vector-Jacobian products on the
 *   left-perturbation tangent spaces: g_pose [n][6], g_ext [n][6], g_X [n][3]
 *   (g2o ordering: rotation first).  Jacobians J_pose [n][2][6],
 *   J_ext [n][2][6], J_X [n][2][3] are written when the pointers are non-NULL.
 * double_precision selects FP64 (1) or FP32 (0) buffers. */
int mcba_reproj_forward(int32_t double_precision, int64_t n, const void* pose_qt, const void* ext_qt,
                        const void* pose_delta, const void* ext_delta, const void* X, const void* K,
                        const void* obs, void* res, void* stream);
int mcba_reproj_backward(int32_t double_precision, int64_t n, const void* pose_qt, const void* ext_qt,
                         const void* pose_delta, const void* ext_delta, const void* X, const void* K,
                         const void* grad_res, void* g_pose, void* g_ext, void* g_X, void* J_pose,
                         void* J_ext, void* J_X, void* stream);

/* ------------------------------------------------ device measurement -- */
/* No counterpart in the reference: the FP64 FMA rate of `device` in
 * GFLOP/s, measured with a saturating FMA kernel (CUDA events, best of five
 * launches).  The roofline of the FP64 factorisation kernels is stated
 * against it. */
int mcba_fp64_fma_rate(int32_t device, double* gflops);

/* ----------------------------------------- allocation-free robust cost -- */
/* No counterpart in the reference: there every optimiser call allocates.
 * Sum of rho(e' Omega e) (the quantity of activeRobustChi2) over n mono edges
 * already in device memory, for callers that must not allocate device memory
 * -- a tracking thread with a hard per-frame deadline (cudaMalloc/cudaFree can
 * wait for the whole device) or an application whose own pool owns all device
 * memory.  Its scratch is a fixed 32 KB file-scope device array shared by all
 * calls on a device: n is limited to MCBA_NOALLOC_MAX_EDGES (larger n returns
 * MCBA_ERR_TOO_LARGE) and calls that overlap on the GPU race on the array.
 * The first call on a device looks the array's device address up; make that
 * call before any stream capture on the device.  The address it keeps is that
 * of the device's context at the time: after cudaDeviceReset of a device, make
 * no further call on that device in the same process.  A CUDA error already
 * pending on the calling thread is left in place and the call returns
 * MCBA_ERR_CUDA without launching.
 * Inputs (device pointers): pose_qt [n][7] T_body_world, ext_qt [n][7]
 * T_cam_body, X [n][3], K [n][4], obs [n][2], info [n] (NULL: 1), delta [n]
 * Huber threshold (NULL or <= 0: no kernel), robust [n] (NULL: all robust).
 * Output: *cost, one device double.  stream is a cudaStream_t or NULL. */
#define MCBA_NOALLOC_MAX_EDGES (4096 * 256)
int mcba_robust_cost_noalloc(int64_t n, const double* pose_qt, const double* ext_qt, const double* X,
                             const double* K, const double* obs, const double* info, const double* delta,
                             const uint8_t* robust, double* cost, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* MCBA_H */
