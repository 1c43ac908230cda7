// Host-side use of the BAoptimizer shim (no GPU needed): graph building,
// bookkeeping and read-back in the reference's call order
// (include/PoseEstimation.hpp:40-101).
#include <cmath>
#include <cstdio>
#include <memory>

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

int main() {
  mcba::BAoptimizer<KeyFrame, MapPointRef, KFAccess, MPAccess> op(KFAccess{}, MPAccess{});
  if (op.status()) return 10;
  const float K[4] = {500.f, 500.f, 320.f, 240.f};
  const float I4[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
  const int cam = op.addCamera(K, 0.f, I4);
  if (cam != 0) return 11;
  Frame f0{0, {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1}};
  Frame f1{1, {1, 0, 0, -0.3f, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1}};
  op.addKeyFrame(&f0, true);
  op.addKeyFrame(&f1);
  op.addKeyFrame(&f1);  // second insertion is ignored, as in the reference
  std::vector<MapPointRef> pts;
  for (int i = 0; i < 20; ++i) {
    auto p = std::make_shared<Point>(Point{{-1.f + 0.1f * i, 0.5f, 5.f + 0.05f * i}});
    pts.push_back(p);
    op.addMapppint(p, false);
    for (KeyFrame kf : {&f0, &f1}) {
      const float x = p->X[0] + kf->T[3], y = p->X[1], z = p->X[2];
      if (op.addEdge(kf, p, cam, 500.f * x / z + 320.f, 500.f * y / z + 240.f, 1.f)) return 12;
    }
  }
  if (op.getEdgeSize() != 40 || op.KF2ID.size() != 2 || op.MP2ID.size() != 20) return 13;
  float T[16], X[3];
  if (op.eval(&f1, T) || std::fabs(T[3] + 0.3f) > 1e-7f) return 14;
  if (op.eval(pts[3], X) || X[2] != pts[3]->X[2]) return 15;
  int n = 0;
  op.filter([&](auto& info) {
    if (info.edge.level() == 0) ++n;
    if (info.edge.id % 5 == 0) info.edge.setLevel(1);
  });
  if (n != 40) return 16;
  std::printf("shim ok\n");
  return 0;
}
