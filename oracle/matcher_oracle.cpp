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

}  // extern "C"
