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

#include <algorithm>
#include <climits>
#include <cmath>
#include <utility>
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

// Frame::ComputeStereoMatch (src/Frame.cpp:150-325) over a batch of stereo
// frames, restated literally: the row table of right keypoints (band of
// 10 * mvScaleFactor[octave] rows around each), per left keypoint the
// candidates of its row within one octave and the disparity range, KnnMatch
// k = 2 with FilterRatio(0.70) and FilterThreshold(int(46 * 0.75) = 34), the
// 11 x 11 SAD of centre-subtracted patches over 11 offsets at the keypoint's
// pyramid level, parabola sub-pixel fit, disparity test, and the median
// filter of the best SAD distances.  Pyramids: per frame one byte buffer of
// pyr_bytes, level l row-major at level_offset[l], level_rows[l] x
// level_cols[l].  Outputs u_right and depth per left keypoint (-1: none).
// Where the reference reads outside its arrays, this restatement defines the
// result: rows of the band outside [0, image_rows) are dropped, a left
// keypoint whose row is outside the table has no candidates, a right window
// starting left of column 0 skips the keypoint (OpenCV would throw), and a
// frame without matches skips the median filter (the reference indexes an
// empty vector).
void orc_stereo_match(int32_t n_threads, int32_t n_frames, int32_t n_levels, const float* scale,
                      const float* inv_scale, const int32_t* level_rows, const int32_t* level_cols,
                      const int64_t* level_offset, int64_t pyr_bytes, const uint8_t* left_pyr,
                      const uint8_t* right_pyr, int32_t image_rows, float b, float bf, const int32_t* left_begin,
                      const float* left_xy, const int32_t* left_oct, const uint8_t* left_desc,
                      const int32_t* right_begin, const float* right_xy, const int32_t* right_oct,
                      const uint8_t* right_desc, float* u_right, float* depth) {
  (void)n_levels;
#pragma omp parallel for num_threads(n_threads > 0 ? n_threads : 1) schedule(dynamic, 1) if (n_threads > 1)
  for (int32_t f = 0; f < n_frames; ++f) {
    const int32_t l0 = left_begin[f], nl = left_begin[f + 1] - l0;
    const int32_t r0 = right_begin[f], nr = right_begin[f + 1] - r0;
    const uint8_t* LP = left_pyr + (size_t)f * pyr_bytes;
    const uint8_t* RP = right_pyr + (size_t)f * pyr_bytes;
    float* ur = u_right + l0;
    float* dp = depth + l0;
    for (int i = 0; i < nl; ++i) {
      ur[i] = -1.0f;
      dp[i] = -1.0f;
    }
    const int nRows = image_rows;
    std::vector<std::vector<int>> rows((size_t)nRows);
    for (int iR = 0; iR < nr; ++iR) {
      const float kpY = right_xy[2 * (size_t)(r0 + iR) + 1];
      const float r = 10.f * scale[right_oct[r0 + iR]];
      const int maxr = (int)std::ceil(kpY + r);
      const int minr = (int)std::floor(kpY - r);
      for (int yi = std::max(minr, 0); yi <= std::min(maxr, nRows - 1); ++yi) rows[yi].push_back(iR);
    }
    const float minZ = b;
    const float minD = 1;
    const float maxD = std::min(bf / minZ, float(1000.0));
    std::vector<std::pair<int, int>> vDistIdx;
    for (int iL = 0; iL < nl; ++iL) {
      const int levelL = left_oct[l0 + iL];
      const float vL = left_xy[2 * (size_t)(l0 + iL) + 1];
      const float uL = left_xy[2 * (size_t)(l0 + iL)];
      if (!(vL >= 0) || (size_t)vL >= (size_t)nRows) continue;
      const std::vector<int>& cands = rows[(size_t)vL];
      if (cands.empty()) continue;
      const float minU = uL - maxD;
      const float maxU = uL - minD;
      if (maxU < 0) continue;
      std::vector<int> cand;
      for (int iR : cands) {
        const int o = right_oct[r0 + iR];
        if (o < levelL - 1 || o > levelL + 1) continue;
        const float uR = right_xy[2 * (size_t)(r0 + iR)];
        if (uR >= minU && uR <= maxU) cand.push_back(iR);
      }
      if (cand.empty()) continue;
      const uint32_t* q = reinterpret_cast<const uint32_t*>(left_desc + 32 * (size_t)(l0 + iL));
      unsigned d[2] = {999, 999};
      unsigned di[2] = {0, 0};
      for (size_t j = 0; j < cand.size(); ++j) {
        const unsigned dj = hamming(q, reinterpret_cast<const uint32_t*>(right_desc + 32 * (size_t)(r0 + cand[j])));
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
      if (!((float)d[0] / (float)d[1] <= 0.70f)) continue;
      if ((float)d[0] > (float)(int)(46 * 0.75)) continue;
      const float uR0 = right_xy[2 * (size_t)(r0 + cand[di[0]])];
      const float scaleFactor = inv_scale[levelL];
      const float scaleduL = std::round(uL * scaleFactor);
      const float scaledvL = std::round(vL * scaleFactor);
      const float scaleduR0 = std::round(uR0 * scaleFactor);
      const int w = 5;
      const int rowsL = level_rows[levelL], colsL = level_cols[levelL];
      if (scaledvL - w < 0 || scaledvL + w + 1 >= rowsL || scaleduL - w < 0 || scaleduL + w + 1 >= colsL) continue;
      const uint8_t* imL = LP + level_offset[levelL];
      const uint8_t* imR = RP + level_offset[levelL];
      const int yv = (int)scaledvL, xl = (int)scaleduL, xr = (int)scaleduR0;
      short IL[11][11];
      for (int rr = 0; rr < 11; ++rr)
        for (int cc = 0; cc < 11; ++cc) IL[rr][cc] = (short)imL[(size_t)(yv - w + rr) * colsL + (xl - w + cc)];
      const short cL = IL[w][w];
      for (int rr = 0; rr < 11; ++rr)
        for (int cc = 0; cc < 11; ++cc) IL[rr][cc] = (short)(IL[rr][cc] - cL);
      int bestDist = INT_MAX;
      int bestincR = 0;
      const int L = 5;
      float vDists[2 * L + 1];
      const float iniu = scaleduR0 + L - w;
      const float endu = scaleduR0 + L + w + 1;
      if (iniu < 0 || endu >= colsL) continue;
      if (xr - L - w < 0) continue;  // the reference's colRange would throw here
      for (int incR = -L; incR <= +L; ++incR) {
        const int x0 = xr + incR - w;
        const short cR = (short)imR[(size_t)yv * colsL + (xr + incR)];
        double acc = 0.0;
        for (int rr = 0; rr < 11; ++rr)
          for (int cc = 0; cc < 11; ++cc) {
            const short vR = (short)((short)imR[(size_t)(yv - w + rr) * colsL + (x0 + cc)] - cR);
            acc += std::abs((int)IL[rr][cc] - (int)vR);
          }
        const float dist = (float)acc;
        if (dist < bestDist) {
          bestDist = (int)dist;
          bestincR = incR;
        }
        vDists[L + incR] = dist;
      }
      if (bestincR == -L || bestincR == L) continue;
      const float dist1 = vDists[L + bestincR - 1];
      const float dist2 = vDists[L + bestincR];
      const float dist3 = vDists[L + bestincR + 1];
      const float deltaR = (dist1 - dist3) / (2.0f * (dist1 + dist3 - 2.0f * dist2));
      if (deltaR < -1 || deltaR > 1) continue;
      const float bestuR = scale[levelL] * ((float)scaleduR0 + (float)bestincR + deltaR);
      const float disparity = (uL - bestuR);
      if (disparity >= minD && disparity < maxD) {
        dp[iL] = bf / disparity;
        ur[iL] = bestuR;
        vDistIdx.push_back(std::pair<int, int>(bestDist, iL));
      }
    }
    if (vDistIdx.empty()) continue;
    std::sort(vDistIdx.begin(), vDistIdx.end());
    const float median = vDistIdx[vDistIdx.size() * 1.0 / 2].first;
    const float th_max_dist = 1.6f * median;
    const float th_min_dist = 0.4 * median;
    int l = 0, r = (int)vDistIdx.size() - 1;
    for (; r >= 0 && vDistIdx[r].first > th_max_dist; r--) {
      ur[vDistIdx[r].second] = -1;
      dp[vDistIdx[r].second] = -1;
    }
    for (; l < r && vDistIdx[l].first < th_min_dist; l++) {
      ur[vDistIdx[l].second] = -1;
      dp[vDistIdx[l].second] = -1;
    }
  }
}

}  // extern "C"
