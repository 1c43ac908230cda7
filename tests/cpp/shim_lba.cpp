// End-to-end use of the BAoptimizer shim on the GPU, in the order of
// PoseEstimation::BoundleAdjustment (include/PoseEstimation.hpp:35-119 of the
// reference): keyframes, map points and edges added one by one through the
// shim, optimize(n), the chi2 filter of FilterCallBack_Chi2
// (src/PoseEstimation.cpp:132-151) through filter(), and recovery_all.
//
// Input (argv[1], written by tests/test_cpp_shim.py): int32 n_cams, n_poses,
// n_points, n_edges, iterations; float chi2 threshold; per camera K[4], bf,
// T_cam_body[16]; per keyframe T[16] and a fixed byte; per map point X[3] and
// a fixed byte; per edge type byte, pose, point, camera (int32), u, v, u_right,
// information (float).
// Output (argv[2]): int32 return value, written flag, last status; the edge
// levels (bytes); the recovered keyframe poses (16 floats each) and map
// points (3 floats each).
#include <cstdint>
#include <cstdio>
#include <memory>
#include <vector>

#include "mcba_baoptimizer.hpp"

struct Frame {
  int id;
  float T[16];
};
struct Point {
  float X[3];
};
using KeyFrame = Frame*;
using MapPointRef = std::shared_ptr<Point>;

struct KFAccess {
  void pose(const KeyFrame& kf, float T[16]) const {
    for (int i = 0; i < 16; ++i) T[i] = kf->T[i];
  }
  bool fixed_id0(const KeyFrame& kf) const { return kf->id == 0; }
};
struct MPAccess {
  void pos(const MapPointRef& mp, float X[3]) const {
    for (int i = 0; i < 3; ++i) X[i] = mp->X[i];
  }
};

template <typename T>
static bool rd(FILE* f, T* v, size_t n = 1) {
  return std::fread(v, sizeof(T), n, f) == n;
}

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 3;
  int32_t hdr[5];
  float thr = 0.f;
  if (!rd(f, hdr, 5) || !rd(f, &thr)) return 4;
  const int n_cams = hdr[0], n_poses = hdr[1], n_points = hdr[2], n_edges = hdr[3], iters = hdr[4];

  mcba::BAoptimizer<KeyFrame, MapPointRef, KFAccess, MPAccess> op(KFAccess{}, MPAccess{});
  if (op.status()) return 10;
  for (int c = 0; c < n_cams; ++c) {
    float K[4], bf, Tcb[16];
    if (!rd(f, K, 4) || !rd(f, &bf) || !rd(f, Tcb, 16)) return 5;
    if (op.addCamera(K, bf, Tcb) != c) return 11;
  }
  std::vector<Frame> frames(n_poses);
  std::vector<uint8_t> pose_fixed(n_poses);
  for (int i = 0; i < n_poses; ++i) {
    frames[i].id = i;
    if (!rd(f, frames[i].T, 16) || !rd(f, &pose_fixed[i])) return 6;
  }
  std::vector<MapPointRef> points(n_points);
  std::vector<uint8_t> point_fixed(n_points);
  for (int i = 0; i < n_points; ++i) {
    points[i] = std::make_shared<Point>();
    if (!rd(f, points[i]->X, 3) || !rd(f, &point_fixed[i])) return 7;
  }
  // vertices in id order, so the shim's ids equal the file's indices
  for (int i = 0; i < n_poses; ++i)
    if (op.addKeyFrame(&frames[i], pose_fixed[i] != 0)) return 12;
  for (int i = 0; i < n_points; ++i)
    if (op.addMapppint(points[i], point_fixed[i] != 0)) return 13;
  for (int e = 0; e < n_edges; ++e) {
    uint8_t type;
    int32_t pose, point, cam;
    float obs[3], info;
    if (!rd(f, &type) || !rd(f, &pose) || !rd(f, &point) || !rd(f, &cam) || !rd(f, obs, 3) || !rd(f, &info))
      return 8;
    int rc;
    if (type == 1)
      rc = op.addEdgeStereo(&frames[pose], points[point], cam, obs[0], obs[1], obs[2], info);
    else if (cam == 0)
      rc = op.addEdge(&frames[pose], points[point], cam, obs[0], obs[1], info);
    else
      rc = op.addEdgeToBody(&frames[pose], points[point], cam, obs[0], obs[1], info);
    if (rc) return 14;
  }
  std::fclose(f);

  op.optimize(iters);
  const int status_opt = op.status();

  // BoundleAdjustment's filter stage.  The reference hands the raw callback to
  // filter(), so its nBad counter never moves and the return value is the
  // edge count (include/PoseEstimation.hpp:103-118).
  const int init_cnt = op.getEdgeSize();
  const int nBad = 0;
  op.filter([&](auto& info) -> bool {
    if (info.edge.level() == 1) return false;
    info.edge.computeError();
    const float chi2 = (float)info.edge.chi2();
    if (chi2 >= thr) {
      info.edge.setLevel(1);
      return true;
    }
    return false;
  });
  const int success = init_cnt - nBad;
  int written = 0;
  std::vector<float> T_out((size_t)n_poses * 16, 0.f), X_out((size_t)n_points * 3, 0.f);
  if (success > 10) {
    op.recovery_all([&](const KeyFrame& kf, const float* T) {
                      for (int k = 0; k < 16; ++k) T_out[(size_t)kf->id * 16 + k] = T[k];
                    },
                    [&](const MapPointRef& mp, const float* X) {
                      for (int k = 0; k < 3; ++k) mp->X[k] = X[k];  // mp->SetWorldPos
                    });
    written = 1;
  }
  for (int i = 0; i < n_points; ++i)
    for (int k = 0; k < 3; ++k) X_out[(size_t)i * 3 + k] = points[i]->X[k];
  std::vector<uint8_t> levels(n_edges, 0);
  op.filter([&](auto& info) -> bool {
    levels[info.edge.id] = (uint8_t)info.edge.level();
    return false;
  });

  FILE* o = std::fopen(argv[2], "wb");
  if (!o) return 9;
  const int32_t head[3] = {success, written, status_opt};
  std::fwrite(head, sizeof(int32_t), 3, o);
  std::fwrite(levels.data(), 1, levels.size(), o);
  std::fwrite(T_out.data(), sizeof(float), T_out.size(), o);
  std::fwrite(X_out.data(), sizeof(float), X_out.size(), o);
  std::fclose(o);
  std::printf("shim lba ok\n");
  return 0;
}
