// matcher_oracle.cpp -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
//
// CPU restatement of MCVSLAM's brute-force Hamming k-nearest-neighbour match
// (Matcher::KnnMatch over descriptor lists, src/Matcher.cpp:245-302, with
// HammingDistance of include/Matcher.hpp:19-31) and of the filters its
// callers apply (MatchResKnn::FilterRatio, src/Matcher.cpp:100-111, default
// ratio 0.6; MatchRes::FilterThreshold, src/Matcher.cpp:23-34, default
// ORB_GOOD_THRESHOLD = 46).  Used only by the tests and the benchmark's CPU
// legs.  Parity status: unpinned (the reference ships no fixtures for it and
// cannot be built here); it follows the cited source line by line.

#include <stdint.h>

#include <cmath>
#include <unordered_map>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// Matcher.hpp:19-31: eight 32-bit words, SWAR population count per word.
inline unsigned hamming(const uint32_t* a, const uint32_t* b) {
  unsigned dist = 0;
  for (int i = 0; i < 8; ++i) {
    unsigned v = a[i] ^ b[i];
    v = v - ((v >> 1) & 0x55555555u);
    v = (v & 0x33333333u) + ((v >> 2) & 0x33333333u);
    dist += (((v + (v >> 4)) & 0xF0F0F0Fu) * 0x1010101u) >> 24;
  }
  return dist;
}

}  // namespace

extern "C" {

// For every query i: the best and second-best train index and distance in
// the reference's loop order (strict '<', so the earliest index wins ties),
// starting from d = {999, 999}, idx = {0, 0} (src/Matcher.cpp:257-271, KnnMatch at 283-302).
// keep[i] (optional) = FilterRatio(ratio) && FilterThreshold(max_dist).
void orc_knn_hamming(const uint8_t* query, int32_t nq, const uint8_t* train, int32_t nt, int32_t* idx, int32_t* dist,
                     float ratio, int32_t max_dist, uint8_t* keep, int32_t n_threads) {
#pragma omp parallel for num_threads(n_threads > 0 ? n_threads : 1) schedule(static) if (n_threads > 1)
  for (int32_t i = 0; i < nq; ++i) {
    const uint32_t* q = reinterpret_cast<const uint32_t*>(query + 32 * (size_t)i);
    unsigned d[2] = {999, 999};
    unsigned di[2] = {0, 0};
    for (int32_t j = 0; j < nt; ++j) {
      const unsigned dj = hamming(q, reinterpret_cast<const uint32_t*>(train + 32 * (size_t)j));
      if (dj < d[0]) {
        d[1] = d[0];
        di[1] = di[0];
        d[0] = dj;
        di[0] = (unsigned)j;
      } else if (dj < d[1]) {
        d[1] = dj;
        di[1] = (unsigned)j;
      }
    }
    idx[2 * (size_t)i] = (int32_t)di[0];
    idx[2 * (size_t)i + 1] = (int32_t)di[1];
    dist[2 * (size_t)i] = (int32_t)d[0];
    dist[2 * (size_t)i + 1] = (int32_t)d[1];
    if (keep) {
      // DMatch distances are float: d0 / d1 <= ratio (0 / 0 is NaN: dropped)
      const float r = (float)d[0] / (float)d[1];
      keep[i] = (r <= ratio && (float)d[0] <= (float)max_dist) ? 1 : 0;
    }
  }
}

// Object::ProjectBunchMapPoints (src/Object.cpp:208-236) over a batch of
// objects, each with its own pose, pinhole camera, keypoint grid and list of
// map points in visit order.  Restated literally:
//  * the grid (Object::AssignFeaturesToGrid / PosInGrid, src/Object.cpp:182-201,
//    250-257): 30 x 30 cells, cell = round(x * 30 / cols), keypoints outside
//    [0, 30) dropped, cells filled in keypoint order;
//  * Pc = R * X + t as OpenCV evaluates the expression `R * X + t` on CV_32F
//    matrices (one gemm call: float products summed in double in k order, the
//    added matrix folded in in double, one rounding to float -- OpenCV 4.x
//    GEMMSingleMul with a double work type; OpenCV is not part of the
//    reference tree);
//  * Pinhole::project (modules/camera/Pinhole.cpp:45-47) in float;
//  * r = r_threshold * mvScaleFactor[level] and GetFeaturesInArea
//    (src/Object.cpp:263-300) with its cell loops;
//  * KnnMatch of the one map-point descriptor against the candidates, then
//    FilterRatio / FilterThreshold (src/Object.cpp:226);
//  * AddMapPoint (src/Object.cpp:113-137) with its two DelMapPoint calls on the
//    keypoint -> map point binding kp_bind (object-local, -1 = none) and the
//    inverse map rebuilt from it.
// mp_match[m] = the keypoint the map point matched (-1 none); obj_count[o] =
// the returned count.  Level indices must be valid.  Objects are independent:
// n_threads > 1 spreads them over OpenMP threads (the reference's loop is
// serial within an object).
void orc_project_match(int32_t n_threads, int32_t n_objects, const float* obj_Rt, const float* obj_K, const int32_t* obj_size,
                       const float* obj_radius, const float* obj_scale, int32_t n_levels, float ratio,
                       int32_t max_dist, const int32_t* kp_begin, const float* kp_xy, const uint8_t* kp_desc,
                       const int32_t* mp_begin, const float* mp_X, const uint8_t* mp_desc, const int32_t* mp_level,
                       const int32_t* mp_id, int32_t* kp_bind, int32_t* mp_match, int32_t* obj_count) {
  const int kCols = 30, kRows = 30;
#pragma omp parallel for num_threads(n_threads > 0 ? n_threads : 1) schedule(dynamic, 1) if (n_threads > 1)
  for (int32_t o = 0; o < n_objects; ++o) {
    const float* Rt = obj_Rt + 12 * (size_t)o;
    const float* K = obj_K + 4 * (size_t)o;
    const int cols = obj_size[2 * o], rows = obj_size[2 * o + 1];
    const double inv_w = static_cast<double>((unsigned)kCols) / cols;
    const double inv_h = static_cast<double>((unsigned)kRows) / rows;
    const int32_t k0 = kp_begin[o], nk = kp_begin[o + 1] - k0;
    std::vector<std::vector<int>> grid((size_t)kCols * kRows);
    for (int i = 0; i < nk; ++i) {
      const float x = kp_xy[2 * (size_t)(k0 + i)], y = kp_xy[2 * (size_t)(k0 + i) + 1];
      const int px = (int)std::round((x - 0) * inv_w);
      const int py = (int)std::round((y - 0) * inv_h);
      if (px < 0 || px >= kCols || py < 0 || py >= kRows) continue;
      grid[(size_t)px * kRows + py].push_back(i);
    }
    std::unordered_map<int32_t, int32_t> mp2idx;
    int32_t* bind = kp_bind + k0;
    for (int i = 0; i < nk; ++i)
      if (bind[i] >= 0) mp2idx[bind[i]] = i;
    int32_t cnt = 0;
    for (int32_t m = mp_begin[o]; m < mp_begin[o + 1]; ++m) {
      mp_match[m] = -1;
      const float* X = mp_X + 3 * (size_t)m;
      float Pc[3];
      for (int r = 0; r < 3; ++r) {
        double s = 0.0;
        for (int k = 0; k < 3; ++k) s += (double)Rt[3 * r + k] * (double)X[k];
        Pc[r] = (float)(s * 1.0 + 1.0 * (double)Rt[9 + r]);
      }
      if (Pc[2] < 0) continue;
      const float u = K[0] * Pc[0] / Pc[2] + K[2];
      const float v = K[1] * Pc[1] / Pc[2] + K[3];
      const float rad = obj_radius[o] * obj_scale[(size_t)o * n_levels + mp_level[m]];
      // GetFeaturesInArea
      std::vector<int> cand;
      if (!(u < 0 || v < 0 || u >= cols || v >= rows) && !std::isnan(u) && !std::isnan(v)) {
        const int minx = std::max(0, (int)std::floor((u - 0 - rad) * inv_w));
        const int maxx = std::min(kCols - 1, (int)std::ceil((u - 0 + rad) * inv_w));
        const int miny = std::max(0, (int)std::floor((v - 0 - rad) * inv_h));
        const int maxy = std::min(kRows - 1, (int)std::ceil((v - 0 + rad) * inv_h));
        if (minx < kCols && maxx >= 0 && miny < kRows && maxy >= 0) {
          for (int ix = minx; ix <= maxx; ++ix)
            for (int iy = miny; iy <= maxy; ++iy)
              for (int i : grid[(size_t)ix * kRows + iy]) {
                const float dx = kp_xy[2 * (size_t)(k0 + i)] - u;
                const float dy = kp_xy[2 * (size_t)(k0 + i) + 1] - v;
                if (std::fabs(dx) < rad && std::fabs(dy) < rad) cand.push_back(i);
              }
        }
      }
      if (cand.empty()) continue;
      const uint32_t* q = reinterpret_cast<const uint32_t*>(mp_desc + 32 * (size_t)m);
      unsigned d[2] = {999, 999};
      unsigned di[2] = {0, 0};
      for (size_t j = 0; j < cand.size(); ++j) {
        const unsigned dj = hamming(q, reinterpret_cast<const uint32_t*>(kp_desc + 32 * (size_t)(k0 + cand[j])));
        if (dj < d[0]) {
          d[1] = d[0];
          di[1] = di[0];
          d[0] = dj;
          di[0] = (unsigned)j;
        } else if (dj < d[1]) {
          d[1] = dj;
          di[1] = (unsigned)j;
        }
      }
      if (!((float)d[0] / (float)d[1] <= ratio) || (float)d[0] > (float)max_dist) continue;
      const int idx = cand[di[0]];
      // AddMapPoint: DelMapPoint(pMP), DelMapPoint(idx), bind
      auto it = mp2idx.find(mp_id[m]);
      if (it != mp2idx.end()) {
        bind[it->second] = -1;
        mp2idx.erase(it);
      }
      if (bind[idx] >= 0) {
        mp2idx.erase(bind[idx]);
        bind[idx] = -1;
      }
      bind[idx] = mp_id[m];
      mp2idx[mp_id[m]] = idx;
      mp_match[m] = idx;
      ++cnt;
    }
    obj_count[o] = cnt;
  }
}

}  // extern "C"
