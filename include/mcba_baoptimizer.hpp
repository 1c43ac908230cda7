// mcba_baoptimizer.hpp -- header-only C++ shim with the method names of
// MCVSLAM::BAoptimizer (include/BAoptimizer.hpp:29-80 of the reference) over
// the C ABI of libmcba.so (mcba.h).
//
// The reference keys vertices by KeyFrame (Frame*) and MapPointRef
// (shared_ptr<MapPoint>) and reads their poses and cameras through OpenCV
// matrices.  The shim is templated on those handle types and takes the
// numbers through small accessor functors, so it has no OpenCV, g2o or
// Eigen dependency; a caller passes adapters such as
//
//   struct KFAccess {                       // for MCVSLAM::KeyFrame
//     void pose(const KeyFrame& kf, float T[16]) const;   // kf->GetPose()
//     bool fixed_id0(const KeyFrame& kf) const;           // kf->id == 0
//   };
//   struct MPAccess {                       // for MCVSLAM::MapPointRef
//     void pos(const MapPointRef& mp, float X[3]) const;  // mp->GetWorldPos()
//   };
//
// Every call reports failures by exception-free status codes (MCBA_*),
// matching the reference's assert-only error behaviour with explicit
// returns instead.
#pragma once

#include <cstdint>
#include <functional>
#include <limits>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "mcba.h"

namespace mcba {

template <typename KeyFrame, typename MapPointRef, typename KFAccess, typename MPAccess,
          typename KFHash = std::hash<KeyFrame>, typename MPHash = std::hash<MapPointRef>>
class BAoptimizer {
 public:
  // One edge of the graph as the filter callbacks see it
  // (BAoptimizer::EdgeInfoMation, include/BAoptimizer.hpp:67-68).
  struct Edge {
    BAoptimizer* opt;
    int32_t id;
    int level() const { return opt->levels_[id]; }
    void setLevel(int lv) { opt->levels_[id] = (uint8_t)lv; opt->dirty_levels_ = true; }
    void computeError() { opt->refresh_chi2(); }
    // g2o's chi2() returns the value of the last computeError(); here the
    // per-edge values are evaluated on first use after optimize()/filter()
    // at the current estimates, so chi2() is valid without a prior
    // computeError().  NaN if the evaluation failed (see status()).
    double chi2() {
      opt->refresh_chi2();
      return opt->chi2_ok_ ? opt->chi2_[id] : std::numeric_limits<double>::quiet_NaN();
    }
    void setRobustKernel(bool on) { opt->robust_[id] = on ? 1 : 0; opt->dirty_robust_ = true; }
  };
  struct EdgeInfo {
    Edge edge;
    MapPointRef mp;
    int camera;  // the reference stores kf->LEFT for every edge (src/BAoptimizer.cpp:64,87,107)
  };

  BAoptimizer(KFAccess kfa, MPAccess mpa, const mcba_options* opt = nullptr) : kfa_(kfa), mpa_(mpa) {
    status_ = mcba_create(opt, &p_);
  }
  ~BAoptimizer() {
    if (p_) mcba_destroy(p_);
  }
  BAoptimizer(const BAoptimizer&) = delete;
  BAoptimizer& operator=(const BAoptimizer&) = delete;

  int status() const { return status_; }
  const char* lastError() const { return mcba_last_error(p_); }

  // Cameras: K = fx fy cx cy, bf, T_cam_body (float 4x4 row-major).
  int addCamera(const float K[4], float bf, const float Tcb[16]) {
    int32_t id = -1;
    status_ = mcba_add_camera(p_, K, bf, Tcb, &id);
    return status_ ? -1 : id;
  }

  // src/BAoptimizer.cpp:22-31
  int addKeyFrame(const KeyFrame& kf, bool fixed = false) {
    if (KF2ID.count(kf)) return MCBA_OK;
    float T[16];
    kfa_.pose(kf, T);
    int32_t id = -1;
    status_ = mcba_add_keyframe(p_, T, (fixed || kfa_.fixed_id0(kf)) ? 1 : 0, &id);
    if (!status_) {
      KF2ID[kf] = id;
      ALLKFS.push_back(kf);
    }
    return status_;
  }
  // src/BAoptimizer.cpp:33-42
  int addMapppint(const MapPointRef& mp, bool fixed = false) {
    if (MP2ID.count(mp)) return MCBA_OK;
    float X[3];
    mpa_.pos(mp, X);
    int32_t id = -1;
    status_ = mcba_add_mappoint(p_, X, fixed ? 1 : 0, &id);
    if (!status_) {
      MP2ID[mp] = id;
      ALLMPS.push_back(mp);
    }
    return status_;
  }
  // src/BAoptimizer.cpp:45-65 (camera: the left camera with T_cam_body = I)
  int addEdge(const KeyFrame& kf, const MapPointRef& mp, int camera, float u, float v, float invSigma2) {
    return push(mcba_add_edge_mono(p_, KF2ID.at(kf), MP2ID.at(mp), camera, u, v, invSigma2, thHuber2D, nullptr),
                mp, camera);
  }
  // src/BAoptimizer.cpp:67-88
  int addEdgeStereo(const KeyFrame& kf, const MapPointRef& mp, int camera, float u, float v, float ru,
                    float invSigma2) {
    return push(
        mcba_add_edge_stereo(p_, KF2ID.at(kf), MP2ID.at(mp), camera, u, v, ru, invSigma2, thHuber3D, nullptr), mp,
        camera);
  }
  // src/BAoptimizer.cpp:90-108 (camera: the wide camera with T_cam_body = Twl)
  int addEdgeToBody(const KeyFrame& kf, const MapPointRef& mp, int camera, float u, float v, float invSigma2) {
    return push(mcba_add_edge_mono(p_, KF2ID.at(kf), MP2ID.at(mp), camera, u, v, invSigma2, thHuber3D, nullptr),
                mp, camera);
  }

  int getEdgeSize() const {
    int32_t n = 0;
    mcba_edge_count(p_, &n);
    return n;
  }

  // src/BAoptimizer.cpp:110-114
  int optimize(int n, mcba_stats* stats = nullptr) {
    sync_flags();
    chi2_.clear();
    status_ = mcba_optimize(p_, n, stats);
    return status_;
  }
  // src/BAoptimizer.cpp:116-119
  int DumpCalculationGraph(const std::string& file) { return mcba_dump_hessian(p_, file.c_str()); }

  // src/BAoptimizer.cpp:121-132: float 4x4 T_body_world / float[3] world position
  int eval(const KeyFrame& kf, float T[16]) const { return mcba_get_keyframe(p_, KF2ID.at(kf), T); }
  int eval(const MapPointRef& mp, float X[3]) const { return mcba_get_mappoint(p_, MP2ID.at(mp), X); }

  // include/BAoptimizer.hpp:70-73: callback(EdgeInfo&) over every edge
  template <typename Callback>
  void filter(Callback&& cb) {
    chi2_.clear();
    for (auto& info : infos_) cb(info);
    sync_flags();
  }

  // src/BAoptimizer.cpp:134-143 with setters supplied by the caller
  template <typename SetPose, typename SetPos>
  void recovery_all(SetPose&& set_pose, SetPos&& set_pos) const {
    float T[16], X[3];
    for (const auto& kf : ALLKFS)
      if (!eval(kf, T)) set_pose(kf, T);
    for (const auto& mp : ALLMPS)
      if (!eval(mp, X)) set_pos(mp, X);
  }

  std::unordered_map<KeyFrame, int32_t, KFHash> KF2ID;
  std::unordered_map<MapPointRef, int32_t, MPHash> MP2ID;
  std::vector<KeyFrame> ALLKFS;
  std::vector<MapPointRef> ALLMPS;
  // include/BAoptimizer.hpp:62-63 (const float in the reference)
  const float thHuber2D = 2.44744754f;  // sqrt(5.99) rounded to float
  const float thHuber3D = 2.79553223f;  // sqrt(7.815) rounded to float

 private:
  int push(int rc, const MapPointRef& mp, int camera) {
    status_ = rc;
    if (rc) return rc;
    const int32_t id = (int32_t)levels_.size();
    levels_.push_back(0);
    robust_.push_back(1);
    infos_.push_back(EdgeInfo{Edge{this, id}, mp, camera});
    return MCBA_OK;
  }
  void refresh_chi2() {
    if (chi2_.size() == levels_.size()) return;
    sync_flags();
    chi2_.assign(levels_.size(), 0.0);
    chi2_ok_ = true;
    if (!chi2_.empty()) {
      status_ = mcba_edge_chi2(p_, chi2_.data());
      chi2_ok_ = status_ == MCBA_OK;
    }
  }
  void sync_flags() {
    if (dirty_levels_ && !levels_.empty()) mcba_set_edge_levels(p_, levels_.data());
    if (dirty_robust_ && !robust_.empty()) mcba_set_edge_robust(p_, robust_.data());
    dirty_levels_ = dirty_robust_ = false;
  }

  mcba_problem* p_ = nullptr;
  int status_ = MCBA_OK;
  KFAccess kfa_;
  MPAccess mpa_;
  std::vector<uint8_t> levels_, robust_;
  std::vector<double> chi2_;
  bool chi2_ok_ = false;
  std::vector<EdgeInfo> infos_;
  bool dirty_levels_ = false, dirty_robust_ = false;
};

}  // namespace mcba
