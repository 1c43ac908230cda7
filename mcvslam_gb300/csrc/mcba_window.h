// mcba_window.h -- internal interface of the GPU local-BA window assembly
// (mcba_window.cu), used by the C entry mcba_local_window (mcba_api.cpp).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "mcba.h"

namespace mcba {

// The window of one new keyframe and its problem in BAoptimizer insertion
// order (poses: anchors, then the window keyframes; points in first-edge
// order; edges in the insertion loop's order).
struct WindowHost {
  int n_local = 0, n_anchor = 0, n_fixed_points = 0;
  std::vector<uint8_t> kf_role;      // [K] bit 0 optimised, bit 1 anchor
  std::vector<int32_t> pose_kf;      // map keyframe of each pose
  std::vector<uint8_t> pose_fixed;
  std::vector<int32_t> point_mp;     // map point of each point
  std::vector<uint8_t> point_fixed;  // ThisMapPointBeFix
  std::vector<uint8_t> e_type;
  std::vector<int32_t> e_pose, e_point, e_cam;
  std::vector<float> e_obs, e_info, e_delta;
};

// Runs the selection and assembly on `device`; the tables of `map` are host
// arrays, validated by the caller's cheap checks (CSR totals, cur range).
int window_assemble(int device, const mcba_map_desc* map, int32_t cur, int32_t hop, WindowHost& out,
                    std::string* err);
// Frees the cached window workspace of `device` (< 0: every device).
void window_release(int device);

}  // namespace mcba
