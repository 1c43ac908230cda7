// window_oracle.cpp -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
//
// CPU restatement of what Map::AddKeyFrame does before its local bundle
// adjustment (src/Map.cpp:140-145 of the reference) on flat map tables:
//   GrabLocalMap_Mappoint(frame, hop)   src/Map.cpp:730-756
//   GrabAnchorKeyFrames(kfs)            src/Map.cpp:775-796 (with
//                                       GrabLocalMap_EssGraph, :704-728)
//   ThisMapPointBeFix(mp, kfs, fix)     src/PoseEstimation.cpp:153-163
//   the vertex / edge insertion loop of PoseEstimation::BoundleAdjustment
//                                       include/PoseEstimation.hpp:36-97
//   BAoptimizer::addKeyFrame / addMapppint / addEdge / addEdgeStereo /
//   addEdgeToBody                       src/BAoptimizer.cpp:22-108
// It checks the GPU window assembly (mcba_local_window) element for element.
//
// The reference keeps keyframes and map points in std::unordered_set, whose
// iteration order is unspecified.  Here (and in the CUDA path) a set of
// keyframes is walked in ascending map index, and the map points of one
// keyframe object in the order of the observation table; everything else
// follows the reference's loops literally.  Parity is unpinned: the
// reference ships no tests or fixtures for these functions and needs
// OpenCV/ROS to build.

#include <cmath>
#include <cstdint>
#include <set>
#include <unordered_map>
#include <vector>

#include "g2o_oracle.h"

namespace {

constexpr float kMinDisparity = 1.f;  // MIN_DISPARITY, include/PoseEstimation.hpp:14

// Map::GrabLocalMap_Mappoint (src/Map.cpp:730-756)
std::set<int> grab_local_map_mappoint(const orc_map_tables* m, int frame, int hop) {
  hop--;
  std::set<int> ret;
  for (int o = m->obs_begin[frame]; o < m->obs_begin[frame + 1]; ++o) {
    if (m->obs_object[o] != 0) continue;  // frame->LEFT->GetMapPoints()
    const int mp = m->obs_point[o];
    for (int b = m->mp_kf_begin[mp]; b < m->mp_kf_begin[mp + 1]; ++b) ret.insert(m->mp_kf[b]);
  }
  std::set<int> cur_hop = ret;
  while (hop-- > 0 && !cur_hop.empty()) {
    std::set<int> next_hop;
    for (int kf : cur_hop)
      for (int a = m->ess_begin[kf]; a < m->ess_begin[kf + 1]; ++a) {
        const int to = m->ess_adj[a];
        if (!ret.count(to)) {
          ret.insert(to);
          next_hop.insert(to);
        }
      }
    cur_hop = next_hop;
  }
  ret.erase(frame);
  return ret;
}

// Map::GrabAnchorKeyFrames (src/Map.cpp:775-796): the 1-hop essential-graph
// neighbours (GrabLocalMap_EssGraph(kf, 1)) of the smallest-id keyframe that
// have a smaller id still.
std::set<int> grab_anchor_keyframes(const orc_map_tables* m, const std::set<int>& kfs) {
  int kmin = -1;
  for (int kf : kfs)
    if (kmin < 0 || m->kf_id[kmin] > m->kf_id[kf]) kmin = kf;
  if (kmin < 0) return {};
  std::set<int> one_hop;
  for (int a = m->ess_begin[kmin]; a < m->ess_begin[kmin + 1]; ++a) one_hop.insert(m->ess_adj[a]);
  one_hop.erase(kmin);
  std::set<int> anchors;
  for (int kf : one_hop)
    if (m->kf_id[kf] < m->kf_id[kmin]) anchors.insert(kf);
  return anchors;
}

// PoseEstimation::ThisMapPointBeFix (src/PoseEstimation.cpp:153-163)
bool this_map_point_be_fix(const orc_map_tables* m, int mp, const std::set<int>& kfs, const std::set<int>& fix_kfs) {
  unsigned cnt_fix = 0, cnt_no_fix = 0;
  for (int b = m->mp_kf_begin[mp]; b < m->mp_kf_begin[mp + 1]; ++b) {
    const int kf = m->mp_kf[b];
    if (kfs.count(kf))
      cnt_no_fix += 1;
    else if (fix_kfs.count(kf))
      cnt_fix += 1;
  }
  return (cnt_no_fix + 1) * 1. / (cnt_fix + 1) > 1.5 ? false : true;
}

struct Assembler {
  const orc_map_tables* m;
  orc_window_out* out;
  std::unordered_map<int, int> kf2id, mp2id;  // BAoptimizer::KF2ID / MP2ID
  int n_edges = 0;
  bool overflow = false;
  const float th2d = std::sqrt(5.99);   // BAoptimizer::thHuber2D
  const float th3d = std::sqrt(7.815);  // BAoptimizer::thHuber3D

  // BAoptimizer::addKeyFrame (src/BAoptimizer.cpp:22-31): a keyframe already
  // present keeps its first id and fixed flag
  void add_keyframe(int kf, bool fixed) {
    if (kf2id.count(kf)) return;
    const int id = (int)kf2id.size();
    kf2id[kf] = id;
    if (out->pose_kf) out->pose_kf[id] = kf;
    if (out->pose_fixed) out->pose_fixed[id] = (fixed || m->kf_id[kf] == 0) ? 1 : 0;
  }
  // BAoptimizer::addMapppint (src/BAoptimizer.cpp:33-42)
  void add_mappoint(int mp, bool fixed) {
    if (mp2id.count(mp)) return;
    const int id = (int)mp2id.size();
    mp2id[mp] = id;
    if (out->point_mp) out->point_mp[id] = mp;
    if (out->point_fixed) out->point_fixed[id] = fixed ? 1 : 0;
  }
  // addEdge / addEdgeStereo (camera 0: LEFT, T_cam_body = I) and
  // addEdgeToBody (camera 1: WIDE, kf->Twl), src/BAoptimizer.cpp:45-108
  void add_edge(int kf, int o) {
    if (n_edges >= out->max_edges) {
      overflow = true;
      return;
    }
    const int e = n_edges++;
    const bool left = m->obs_object[o] == 0;
    const float ur = m->obs_ur[o];
    const bool stereo = left && ur != -1 && ur >= kMinDisparity;
    const int lv = m->obs_octave[o];
    out->edge_type[e] = stereo ? ORC_EDGE_STEREO : ORC_EDGE_MONO;
    out->edge_pose[e] = kf2id.at(kf);
    out->edge_point[e] = mp2id.at(m->obs_point[o]);
    out->edge_cam[e] = left ? 0 : 1;
    out->edge_obs[3 * e] = m->obs_uv[2 * o];
    out->edge_obs[3 * e + 1] = m->obs_uv[2 * o + 1];
    out->edge_obs[3 * e + 2] = stereo ? ur : 0.f;
    out->edge_info[e] = left ? m->inv_sigma2_left[lv] : m->inv_sigma2_wide[lv];
    out->edge_delta[e] = (left && !stereo) ? th2d : th3d;
  }
  // one keyframe of the insertion loop (include/PoseEstimation.hpp:40-69 and
  // 70-97): its LEFT map points, then its WIDE map points
  void keyframe_block(int kf, bool fixed, const std::set<int>& kfs, const std::set<int>& fix_kfs) {
    add_keyframe(kf, fixed);
    for (int obj = 0; obj < 2; ++obj)
      for (int o = m->obs_begin[kf]; o < m->obs_begin[kf + 1]; ++o) {
        if (m->obs_object[o] != obj) continue;
        const int mp = m->obs_point[o];
        add_mappoint(mp, this_map_point_be_fix(m, mp, kfs, fix_kfs));
        add_edge(kf, o);
      }
  }
};

}  // namespace

extern "C" int orc_local_window(const orc_map_tables* m, int32_t cur, int32_t hop, orc_window_out* out) {
  if (!m || !out || cur < 0 || cur >= m->n_keyframes || hop < 1) return -1;
  // src/Map.cpp:142-144
  std::set<int> local_kfs = grab_local_map_mappoint(m, cur, hop);
  const std::set<int> fix_kfs = grab_anchor_keyframes(m, local_kfs);
  local_kfs.insert(cur);
  if (out->kf_role) {
    for (int k = 0; k < m->n_keyframes; ++k) out->kf_role[k] = 0;
    for (int k : local_kfs) out->kf_role[k] |= 1;
    for (int k : fix_kfs) out->kf_role[k] |= 2;
  }
  // include/PoseEstimation.hpp:36-97
  Assembler a{m, out};
  for (int kf : fix_kfs) a.keyframe_block(kf, true, local_kfs, fix_kfs);
  for (int kf : local_kfs) a.keyframe_block(kf, false, local_kfs, fix_kfs);
  out->n_local = (int32_t)local_kfs.size();
  out->n_anchor = (int32_t)fix_kfs.size();
  out->n_poses = (int32_t)a.kf2id.size();
  out->n_points = (int32_t)a.mp2id.size();
  out->n_edges = a.n_edges;
  return a.overflow ? -2 : 0;
}
