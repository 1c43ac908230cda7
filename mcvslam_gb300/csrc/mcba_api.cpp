// mcba_api.cpp -- C ABI of libmcba.so and the host-side problem compiler.
//
// The entry points mirror MCVSLAM's BAoptimizer (include/BAoptimizer.hpp:29-80)
// and the PoseEstimation drivers; the numeric work runs on the GPU
// (mcba_solver.cu).  Nothing here computes residuals or solves: this file
// converts the caller's float matrices to the FP64 SE3 estimates g2o keeps,
// decides the active set and Hessian ordering exactly as
// initializeOptimization/buildIndexMapping do, and lays the problem out for
// the device kernels.

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "mcba.h"
#include "mcba_host_pool.h"
#include "mcba_internal.h"
#include "mcba_window.h"

namespace mcba {
namespace {

// Rotation matrix (row-major) -> unit quaternion by Shoemake's method, then
// the w >= 0 / unit-norm rule of SE3Quat::normalizeRotation
// (types/slam3d/se3quat.h:53-55,280-285).
QT qt_from_Rt(const double R[9], const double t[3]) {
  QT o;
  double x, y, z, w;
  const double tr = R[0] + R[4] + R[8];
  if (tr > 0) {
    double s = std::sqrt(tr + 1.0);
    w = 0.5 * s;
    s = 0.5 / s;
    x = (R[7] - R[5]) * s;
    y = (R[2] - R[6]) * s;
    z = (R[3] - R[1]) * s;
  } else {
    int i = 0;
    if (R[4] > R[0]) i = 1;
    if (R[8] > R[4 * i]) i = 2;
    const int j = (i + 1) % 3, k = (j + 1) % 3;
    double s = std::sqrt(R[4 * i] - R[4 * j] - R[4 * k] + 1.0);
    double v[3];
    v[i] = 0.5 * s;
    s = 0.5 / s;
    w = (R[3 * k + j] - R[3 * j + k]) * s;
    v[j] = (R[3 * j + i] + R[3 * i + j]) * s;
    v[k] = (R[3 * k + i] + R[3 * i + k]) * s;
    x = v[0];
    y = v[1];
    z = v[2];
  }
  if (w < 0) {
    x = -x;
    y = -y;
    z = -z;
    w = -w;
  }
  const double n = std::sqrt(x * x + y * y + z * z + w * w);
  o.q[0] = x / n;
  o.q[1] = y / n;
  o.q[2] = z / n;
  o.q[3] = w / n;
  o.t[0] = t[0];
  o.t[1] = t[1];
  o.t[2] = t[2];
  return o;
}

// Converter::toSE3Quat (src/Converter.cc:31-39)
QT qt_from_mat44f(const float* M) {
  const double R[9] = {M[0], M[1], M[2], M[4], M[5], M[6], M[8], M[9], M[10]};
  const double t[3] = {M[3], M[7], M[11]};
  return qt_from_Rt(R, t);
}

// Converter::toCvMat(SE3Quat) (src/Converter.cc:41-52)
void qt_to_mat44f(const QT& T, float* M) {
  const double x = T.q[0], y = T.q[1], z = T.q[2], w = T.q[3];
  const double tx = 2 * x, ty = 2 * y, tz = 2 * z;
  const double R[9] = {1 - (ty * y + tz * z), ty * x - tz * w, tz * x + ty * w,
                       ty * x + tz * w,       1 - (tx * x + tz * z), tz * y - tx * w,
                       tz * x - ty * w,       tz * y + tx * w,       1 - (tx * x + ty * y)};
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) M[4 * i + j] = (float)R[3 * i + j];
    M[4 * i + 3] = (float)T.t[i];
  }
  M[12] = M[13] = M[14] = 0.f;
  M[15] = 1.f;
}

bool finite_arr(const float* a, int n) {
  for (int i = 0; i < n; ++i)
    if (!std::isfinite(a[i])) return false;
  return true;
}

constexpr int kChunk = 256;   // edges per linearisation CTA (one pose per chunk)
constexpr int kPairChunk = 128;  // Schur pairs per warp task

}  // namespace

// initializeOptimization (sparse_optimizer.cpp:201-272): active edges are
// level-0 edges with a free vertex; active vertices have an active edge;
// buildIndexMapping (:168-188) numbers free poses, then free points, in id
// order.  buildStructure (block_solver.hpp:103-256) then fixes one Hpl block
// per (pose, point) pair and the Schur pattern from co-observations; here the
// same information becomes the canonical edge order, the per-pose chunk list
// and the list of edge pairs of every reduced-camera block.
bool compile_structure(const HostProblem& hp, Structure& s) {
  const int K = (int)hp.poses.size();
  const int P = (int)hp.point_fixed.size();
  const int Eall = (int)hp.n_edges();
  s = Structure();
  s.K = K;
  s.P = P;
  std::vector<uint8_t> pose_act(K, 0), pt_act(P, 0);
  std::vector<int32_t> act;
  act.reserve(Eall);
  int U = 0;
  for (int i = 0; i < Eall; ++i) {
    if (hp.e_level[i] != 0) continue;
    const bool unary = hp.e_type[i] == MCBA_EDGE_UNARY;
    const bool pf = hp.pose_fixed[hp.e_pose[i]] != 0;
    const bool xf = unary ? true : hp.point_fixed[hp.e_point[i]] != 0;
    if (pf && xf) continue;
    act.push_back(i);
    pose_act[hp.e_pose[i]] = 1;
    if (!unary) pt_act[hp.e_point[i]] = 1;
  }
  for (int i = 0; i < Eall; ++i)
    if (hp.e_type[i] == MCBA_EDGE_UNARY) ++U;
  s.U = U;
  s.pose_h.assign(K, -1);
  s.point_h.assign(P, -1);
  for (int k = 0; k < K; ++k)
    if (pose_act[k] && !hp.pose_fixed[k]) {
      s.pose_h[k] = (int)s.free_pose_ids.size();
      s.free_pose_ids.push_back(k);
    }
  for (int k = 0; k < P; ++k)
    if (pt_act[k] && !hp.point_fixed[k]) {
      s.point_h[k] = (int)s.free_point_ids.size();
      s.free_point_ids.push_back(k);
    }
  s.Kf = (int)s.free_pose_ids.size();
  s.Lf = (int)s.free_point_ids.size();
  s.E = (int)act.size();
  if (s.Kf + s.Lf == 0 || s.E == 0) return false;

  // unary constant points live after the P map points in the state
  std::vector<int32_t> unary_slot(Eall, -1);
  {
    int u = 0;
    for (int i = 0; i < Eall; ++i)
      if (hp.e_type[i] == MCBA_EDGE_UNARY) unary_slot[i] = P + u++;
  }

  // canonical order: edges of free points, by point index then pose index
  const int Lf = s.Lf, Kf = s.Kf;
  std::vector<int32_t> cnt(Lf + 1, 0);
  for (int id : act) {
    if (hp.e_type[id] == MCBA_EDGE_UNARY) continue;
    const int l = s.point_h[hp.e_point[id]];
    if (l >= 0) cnt[l + 1]++;
  }
  for (int l = 0; l < Lf; ++l) cnt[l + 1] += cnt[l];
  s.pt_begin = cnt;
  s.Ec = cnt[Lf];
  std::vector<int32_t> canon_id(s.Ec);
  {
    std::vector<int32_t> fill(cnt.begin(), cnt.end() - 1);
    for (int id : act) {
      if (hp.e_type[id] == MCBA_EDGE_UNARY) continue;
      const int l = s.point_h[hp.e_point[id]];
      if (l >= 0) canon_id[fill[l]++] = id;
    }
  }
  auto ph_of = [&](int id) { return s.pose_h[hp.e_pose[id]]; };
  for (int l = 0; l < Lf; ++l) {
    // insertion sort by (pose index, edge id); fixed poses (-1) first
    for (int a = s.pt_begin[l] + 1; a < s.pt_begin[l + 1]; ++a) {
      const int v = canon_id[a];
      int b = a - 1;
      while (b >= s.pt_begin[l] && (ph_of(canon_id[b]) > ph_of(v) ||
                                    (ph_of(canon_id[b]) == ph_of(v) && canon_id[b] > v))) {
        canon_id[b + 1] = canon_id[b];
        --b;
      }
      canon_id[b + 1] = v;
    }
  }
  std::vector<int32_t> canon_of(Eall, -1);
  s.canon_pose_h.resize(s.Ec);
  s.canon_point_h.resize(s.Ec);
  for (int e = 0; e < s.Ec; ++e) {
    const int id = canon_id[e];
    canon_of[id] = e;
    s.canon_pose_h[e] = ph_of(id);
    s.canon_point_h[e] = s.point_h[hp.e_point[id]];
  }

  // pose-sorted stream: free poses in index order, then fixed-pose edges
  std::vector<int32_t> pcnt(Kf + 2, 0);
  for (int id : act) {
    const int ph = ph_of(id);
    pcnt[(ph >= 0 ? ph : Kf) + 1]++;
  }
  for (int i = 0; i <= Kf; ++i) pcnt[i + 1] += pcnt[i];
  // inside a pose segment: edges of free points in canonical order (locality
  // of the scattered per-edge writes), then the others in id order
  std::vector<int32_t> stream(s.E);
  {
    std::vector<int32_t> fill(pcnt.begin(), pcnt.end() - 1);
    for (int e = 0; e < s.Ec; ++e) {
      const int id = canon_id[e];
      const int ph = ph_of(id);
      stream[fill[ph >= 0 ? ph : Kf]++] = id;
    }
    for (int id : act) {
      if (canon_of[id] >= 0) continue;
      const int ph = ph_of(id);
      stream[fill[ph >= 0 ? ph : Kf]++] = id;
    }
  }
  s.pose_edge_begin.assign(pcnt.begin(), pcnt.begin() + Kf + 1);
  s.recs.resize(s.E);
  s.obs.resize(3 * (size_t)s.E);
  s.active_ids = stream;
  for (int j = 0; j < s.E; ++j) {
    const int id = stream[j];
    EdgeRec& r = s.recs[j];
    const bool unary = hp.e_type[id] == MCBA_EDGE_UNARY;
    r.pose = hp.e_pose[id];
    r.point = unary ? unary_slot[id] : hp.e_point[id];
    r.pose_h = ph_of(id);
    r.point_h = unary ? -1 : s.point_h[hp.e_point[id]];
    r.canon = canon_of[id];
    r.type = hp.e_type[id];
    r.cam = (uint8_t)hp.e_cam[id];
    r.robust = (hp.e_robust[id] && hp.e_delta[id] > 0.f) ? 1 : 0;
    r.dim = (r.type == MCBA_EDGE_STEREO) ? 3 : 2;
    r.info = hp.e_info[id];
    r.delta = hp.e_delta[id];
    for (int d = 0; d < 3; ++d) s.obs[3 * (size_t)j + d] = hp.e_obs[3 * (size_t)id + d];
  }
  // chunks: <= kChunk edges, never spanning two poses
  // the chunks of free pose i are [pose_chunk_begin[i], pose_chunk_begin[i+1]);
  // the fixed-pose chunks follow from pose_chunk_begin[Kf] on (they hold no
  // pose terms, so no reduction may read them)
  s.pose_chunk_begin.assign(Kf + 1, 0);
  for (int i = 0; i <= Kf; ++i) {
    s.pose_chunk_begin[i] = (int)s.chunk_pose.size();
    for (int a = pcnt[i]; a < pcnt[i + 1]; a += kChunk) {
      s.chunk_begin.push_back(a);
      s.chunk_pose.push_back(i < Kf ? i : -1);
    }
  }
  s.chunk_begin.push_back(s.E);

  // canonical edges per free pose (b_schur gather), ascending canonical index
  s.pose_canon_begin.assign(Kf + 1, 0);
  for (int e = 0; e < s.Ec; ++e)
    if (s.canon_pose_h[e] >= 0) s.pose_canon_begin[s.canon_pose_h[e] + 1]++;
  for (int i = 0; i < Kf; ++i) s.pose_canon_begin[i + 1] += s.pose_canon_begin[i];
  s.pose_canon_list.resize(s.pose_canon_begin[Kf]);
  {
    std::vector<int32_t> fill(s.pose_canon_begin.begin(), s.pose_canon_begin.end() - 1);
    for (int e = 0; e < s.Ec; ++e)
      if (s.canon_pose_h[e] >= 0) s.pose_canon_list[fill[s.canon_pose_h[e]]++] = e;
  }

  // Schur pairs (block_solver.hpp:342-393): for every point, every pair of
  // its free-pose edges (i before j in pose order); two edges of one point on
  // the same pose contribute both orders to the diagonal block.
  std::vector<int32_t> blk_of((size_t)Kf * Kf, -1);
  std::vector<int32_t> bab;
  auto visit_pairs = [&](auto&& fn) {
    for (int l = 0; l < Lf; ++l) {
      const int b0 = s.pt_begin[l], b1 = s.pt_begin[l + 1];
      for (int i = b0; i < b1; ++i) {
        const int a = s.canon_pose_h[i];
        if (a < 0) continue;
        for (int j = i; j < b1; ++j) {
          const int b = s.canon_pose_h[j];
          if (b < 0) continue;
          fn(a, b, i, j);
          if (j != i && a == b) fn(a, b, j, i);
        }
      }
    }
  };
  // pairs per reduced-camera block, then block ids in (a, b) lexicographic
  // order (diagonal blocks always exist)
  std::vector<int64_t> pcount((size_t)Kf * Kf, 0);
  visit_pairs([&](int a, int b, int, int) { pcount[(size_t)a * Kf + b]++; });
  std::vector<int64_t> boff(1, 0);
  for (int a = 0; a < Kf; ++a)
    for (int b = a; b < Kf; ++b) {
      const int64_t c = pcount[(size_t)a * Kf + b];
      if (c || a == b) {
        blk_of[(size_t)a * Kf + b] = (int)bab.size() / 2;
        bab.push_back(a);
        bab.push_back(b);
        boff.push_back(boff.back() + c);
      }
    }
  const int nblk = (int)bab.size() / 2;
  const int64_t npairs = boff[nblk];
  s.pair_ij.resize(2 * (size_t)npairs);
  {
    std::vector<int64_t> fill(boff.begin(), boff.end() - 1);
    visit_pairs([&](int a, int b, int i, int j) {
      const int64_t at = fill[blk_of[(size_t)a * Kf + b]]++;
      s.pair_ij[2 * at] = i;
      s.pair_ij[2 * at + 1] = j;
    });
  }
  s.block_ab = bab;
  s.block_chunk_begin.assign(nblk + 1, 0);
  for (int k = 0; k < nblk; ++k) {
    s.block_chunk_begin[k] = (int)s.pchunk_block.size();
    for (int64_t a = boff[k]; a < boff[k + 1]; a += kPairChunk) {
      s.pchunk_begin.push_back((int32_t)a);
      s.pchunk_block.push_back(k);
    }
  }
  s.block_chunk_begin[nblk] = (int)s.pchunk_block.size();
  s.pchunk_begin.push_back((int32_t)npairs);
  return true;
}

}  // namespace mcba

using namespace mcba;

struct mcba_problem {
  mcba_options opt;
  HostProblem hp;
  Structure st;
  bool prepared = false;
  Solver* solver = nullptr;
  std::string err;
  std::vector<mcba_trial_log> log;
  std::vector<double> hpp;
  int hpp_kf = 0;
};

namespace {

int fail(mcba_problem* p, int code, const std::string& msg) {
  if (p) p->err = msg;
  return code;
}

int ensure_solver(mcba_problem* p) {
  if (p->solver) return MCBA_OK;
  std::string e;
  p->solver = solver_create(p->opt.device, p->opt.precision, p->opt.stream, &e);
  if (!p->solver) return fail(p, e.find("no CUDA device") != std::string::npos ? MCBA_ERR_NO_DEVICE : MCBA_ERR_CUDA, e);
  return MCBA_OK;
}

int push_edge(mcba_problem* p, uint8_t type, int32_t kf, int32_t mp, int32_t cam, const float obs[3],
              const float* Xw, float info, float delta, uint8_t robust, uint8_t level) {
  HostProblem& h = p->hp;
  if (type > MCBA_EDGE_UNARY) return fail(p, MCBA_ERR_INVALID, "unknown edge type");
  if (kf < 0 || kf >= (int)h.poses.size()) return fail(p, MCBA_ERR_INVALID, "edge references an unknown keyframe");
  if (type != MCBA_EDGE_UNARY && (mp < 0 || mp >= (int)h.point_fixed.size()))
    return fail(p, MCBA_ERR_INVALID, "edge references an unknown map point");
  if (cam < 0 || cam >= (int)h.cams.size() || cam > 255) return fail(p, MCBA_ERR_INVALID, "edge references an unknown camera");
  if (!finite_arr(obs, 3) || !std::isfinite(info) || !std::isfinite(delta))
    return fail(p, MCBA_ERR_NONFINITE, "non-finite edge measurement");
  if (type == MCBA_EDGE_UNARY && (!Xw || !finite_arr(Xw, 3)))
    return fail(p, MCBA_ERR_NONFINITE, "unary edge needs a finite world point");
  h.e_type.push_back(type);
  h.e_pose.push_back(kf);
  h.e_point.push_back(type == MCBA_EDGE_UNARY ? -1 : mp);
  h.e_cam.push_back(cam);
  for (int d = 0; d < 3; ++d) h.e_obs.push_back(obs[d]);
  h.e_info.push_back(info);
  h.e_delta.push_back(delta);
  h.e_robust.push_back(robust);
  h.e_level.push_back(level);
  if (type == MCBA_EDGE_UNARY)
    for (int d = 0; d < 3; ++d) h.u_Xw.push_back((double)Xw[d]);
  return MCBA_OK;
}

}  // namespace

extern "C" {

int mcba_abi_version(void) { return MCBA_ABI_VERSION; }

const char* mcba_status_string(int s) {
  switch (s) {
    case MCBA_OK: return "ok";
    case MCBA_ERR_INVALID: return "invalid argument";
    case MCBA_ERR_EMPTY: return "nothing to optimise";
    case MCBA_ERR_NOT_PD: return "reduced camera system not positive definite";
    case MCBA_ERR_NONFINITE: return "non-finite input";
    case MCBA_ERR_TIMEOUT: return "device wait timed out";
    case MCBA_ERR_CUDA: return "CUDA error";
    case MCBA_ERR_NOMEM: return "out of memory";
    case MCBA_ERR_NO_DEVICE: return "no CUDA device";
    case MCBA_ERR_TOO_LARGE: return "request above the supported maximum";
    default: return "unknown status";
  }
}

int mcba_release_cached(int32_t device) {
  mcba::solver_release_cached(device);
  mcba::window_release(device);
  return MCBA_OK;
}

void mcba_default_options(mcba_options* o) {
  if (!o) return;
  o->precision = MCBA_PREC_FP64;
  o->device = 0;
  o->tau = 1e-5;
  o->max_trials = 10;
  o->use_graph = 1;
  o->profile = 0;
  o->stream = nullptr;
  o->host_structure = 0;
}

namespace {
// Host-side problem storage of destroyed handles, kept (cleared, with its
// capacity) for the next handle: a caller that creates a handle per solve
// then loads into memory that is already mapped.
std::mutex g_hp_mu;
std::vector<HostProblem> g_hp_pool;
constexpr size_t kHostPoolMax = 64;  // as many as the solver workspaces kept per key
}  // namespace

int mcba_create(const mcba_options* opt, mcba_problem** out) {
  if (!out) return MCBA_ERR_INVALID;
  *out = nullptr;
  mcba_problem* p = new (std::nothrow) mcba_problem();
  if (!p) return MCBA_ERR_NOMEM;
  {
    std::lock_guard<std::mutex> lk(g_hp_mu);
    if (!g_hp_pool.empty()) {
      p->hp = std::move(g_hp_pool.back());
      g_hp_pool.pop_back();
      p->hp.clear();
    }
  }
  if (opt) {
    p->opt = *opt;
  } else {
    mcba_default_options(&p->opt);
  }
  if (p->opt.precision != MCBA_PREC_FP64 && p->opt.precision != MCBA_PREC_MIXED) {
    delete p;
    return MCBA_ERR_INVALID;
  }
  if (p->opt.max_trials <= 0) p->opt.max_trials = 10;
  if (!(p->opt.tau > 0)) p->opt.tau = 1e-5;
  *out = p;
  return MCBA_OK;
}

int mcba_destroy(mcba_problem* p) {
  if (!p) return MCBA_ERR_INVALID;
  if (p->solver) solver_destroy(p->solver);
  {
    std::lock_guard<std::mutex> lk(g_hp_mu);
    if (g_hp_pool.size() < kHostPoolMax) g_hp_pool.push_back(std::move(p->hp));
  }
  delete p;
  return MCBA_OK;
}

const char* mcba_last_error(const mcba_problem* p) { return p ? p->err.c_str() : "null handle"; }

int mcba_clear(mcba_problem* p) {
  if (!p) return MCBA_ERR_INVALID;
  p->hp.clear();
  p->log.clear();
  p->hpp.clear();
  return MCBA_OK;
}

int mcba_add_camera(mcba_problem* p, const float K[4], float bf, const float T[16], int32_t* id) {
  if (!p || !K || !T) return fail(p, MCBA_ERR_INVALID, "null argument");
  if (!finite_arr(K, 4) || !finite_arr(T, 16) || !std::isfinite(bf)) return fail(p, MCBA_ERR_NONFINITE, "non-finite camera");
  if (p->hp.cams.size() >= 255) return fail(p, MCBA_ERR_TOO_LARGE, "at most 255 cameras");
  HostCamera c;
  std::memcpy(c.K, K, sizeof(c.K));
  c.bf = bf;
  c.T_cb = qt_from_mat44f(T);
  p->hp.cams.push_back(c);
  if (id) *id = (int32_t)p->hp.cams.size() - 1;
  return MCBA_OK;
}

int mcba_add_keyframe(mcba_problem* p, const float T[16], int fixed, int32_t* id) {
  if (!p || !T) return fail(p, MCBA_ERR_INVALID, "null argument");
  if (!finite_arr(T, 16)) return fail(p, MCBA_ERR_NONFINITE, "non-finite keyframe pose");
  p->hp.poses.push_back(qt_from_mat44f(T));
  p->hp.pose_fixed.push_back(fixed ? 1 : 0);
  if (id) *id = (int32_t)p->hp.poses.size() - 1;
  return MCBA_OK;
}

int mcba_add_keyframe_qt(mcba_problem* p, const double qt[7], int fixed, int32_t* id) {
  if (!p || !qt) return fail(p, MCBA_ERR_INVALID, "null argument");
  for (int i = 0; i < 7; ++i)
    if (!std::isfinite(qt[i])) return fail(p, MCBA_ERR_NONFINITE, "non-finite keyframe pose");
  QT T;
  double x = qt[0], y = qt[1], z = qt[2], w = qt[3];
  if (w < 0) {
    x = -x;
    y = -y;
    z = -z;
    w = -w;
  }
  const double n = std::sqrt(x * x + y * y + z * z + w * w);
  if (!(n > 0)) return fail(p, MCBA_ERR_INVALID, "zero quaternion");
  T.q[0] = x / n;
  T.q[1] = y / n;
  T.q[2] = z / n;
  T.q[3] = w / n;
  T.t[0] = qt[4];
  T.t[1] = qt[5];
  T.t[2] = qt[6];
  p->hp.poses.push_back(T);
  p->hp.pose_fixed.push_back(fixed ? 1 : 0);
  if (id) *id = (int32_t)p->hp.poses.size() - 1;
  return MCBA_OK;
}

int mcba_add_mappoint(mcba_problem* p, const float X[3], int fixed, int32_t* id) {
  if (!p || !X) return fail(p, MCBA_ERR_INVALID, "null argument");
  if (!finite_arr(X, 3)) return fail(p, MCBA_ERR_NONFINITE, "non-finite map point");
  for (int d = 0; d < 3; ++d) p->hp.points.push_back(X[d]);
  p->hp.point_fixed.push_back(fixed ? 1 : 0);
  if (id) *id = (int32_t)p->hp.point_fixed.size() - 1;
  return MCBA_OK;
}

int mcba_add_edge_mono(mcba_problem* p, int32_t kf, int32_t mp, int32_t cam, float u, float v, float info,
                       float delta, int32_t* id) {
  if (!p) return MCBA_ERR_INVALID;
  const float obs[3] = {u, v, 0.f};
  const int r = push_edge(p, MCBA_EDGE_MONO, kf, mp, cam, obs, nullptr, info, delta, delta > 0.f, 0);
  if (r == MCBA_OK && id) *id = (int32_t)p->hp.n_edges() - 1;
  return r;
}

int mcba_add_edge_stereo(mcba_problem* p, int32_t kf, int32_t mp, int32_t cam, float u, float v, float ur,
                         float info, float delta, int32_t* id) {
  if (!p) return MCBA_ERR_INVALID;
  const float obs[3] = {u, v, ur};
  const int r = push_edge(p, MCBA_EDGE_STEREO, kf, mp, cam, obs, nullptr, info, delta, delta > 0.f, 0);
  if (r == MCBA_OK && id) *id = (int32_t)p->hp.n_edges() - 1;
  return r;
}

int mcba_add_edge_posonly(mcba_problem* p, int32_t kf, int32_t cam, const float Xw[3], float u, float v,
                          float info, float delta, int32_t* id) {
  if (!p) return MCBA_ERR_INVALID;
  const float obs[3] = {u, v, 0.f};
  const int r = push_edge(p, MCBA_EDGE_UNARY, kf, -1, cam, obs, Xw, info, delta, delta > 0.f, 0);
  if (r == MCBA_OK && id) *id = (int32_t)p->hp.n_edges() - 1;
  return r;
}

int mcba_add_edges(mcba_problem* p, int32_t n, const uint8_t* type, const int32_t* kf, const int32_t* mp,
                   const int32_t* cam, const float* obs, const float* Xw, const float* info, const float* delta,
                   int32_t* first_id) {
  if (!p || n < 0 || (n > 0 && (!type || !kf || !cam || !obs))) return fail(p, MCBA_ERR_INVALID, "null argument");
  const size_t before = p->hp.n_edges(), ubefore = p->hp.u_Xw.size();
  if (first_id) *first_id = (int32_t)before;
  for (int32_t i = 0; i < n; ++i) {
    const float inf = info ? info[i] : 1.f;
    const float del = delta ? delta[i] : 0.f;
    const int r = push_edge(p, type[i], kf[i], mp ? mp[i] : -1, cam[i], obs + 3 * (size_t)i,
                            Xw ? Xw + 3 * (size_t)i : nullptr, inf, del, del > 0.f, 0);
    if (r != MCBA_OK) {
      // roll back this call's edges so the graph stays as it was
      HostProblem& h = p->hp;
      h.e_type.resize(before);
      h.e_pose.resize(before);
      h.e_point.resize(before);
      h.e_cam.resize(before);
      h.e_obs.resize(3 * before);
      h.e_info.resize(before);
      h.e_delta.resize(before);
      h.e_robust.resize(before);
      h.e_level.resize(before);
      h.u_Xw.resize(ubefore);
      return r;
    }
  }
  return MCBA_OK;
}

int mcba_load(mcba_problem* p, const mcba_problem_desc* d) {
  if (!p || !d) return fail(p, MCBA_ERR_INVALID, "null argument");
  if (d->n_cams < 0 || d->n_poses < 0 || d->n_points < 0 || d->n_edges < 0)
    return fail(p, MCBA_ERR_INVALID, "negative size");
  if ((d->n_cams && (!d->cam_K || !d->cam_Tcb)) || (d->n_poses && !d->pose_Tcw) ||
      (d->n_points && !d->point_Xw) ||
      (d->n_edges && (!d->edge_type || !d->edge_pose || !d->edge_point || !d->edge_cam || !d->edge_obs)))
    return fail(p, MCBA_ERR_INVALID, "null array");
  mcba_clear(p);
  int r;
  for (int c = 0; c < d->n_cams; ++c)
    if ((r = mcba_add_camera(p, d->cam_K + 4 * c, d->cam_bf ? d->cam_bf[c] : 0.f, d->cam_Tcb + 16 * c, nullptr)))
      return r;
  HostProblem& h = p->hp;
  h.poses.resize(d->n_poses);
  h.pose_fixed.resize(d->n_poses);
  for (int k = 0; k < d->n_poses; ++k) {
    if (!finite_arr(d->pose_Tcw + 16 * (size_t)k, 16)) return fail(p, MCBA_ERR_NONFINITE, "non-finite keyframe pose");
    h.poses[k] = qt_from_mat44f(d->pose_Tcw + 16 * (size_t)k);
    h.pose_fixed[k] = d->pose_fixed ? (d->pose_fixed[k] ? 1 : 0) : 0;
  }
  h.points.resize(3 * (size_t)d->n_points);
  h.point_fixed.resize(d->n_points);
  for (int k = 0; k < d->n_points; ++k) {
    for (int a = 0; a < 3; ++a) {
      const float v = d->point_Xw[3 * (size_t)k + a];
      if (!std::isfinite(v)) return fail(p, MCBA_ERR_NONFINITE, "non-finite map point");
      h.points[3 * (size_t)k + a] = v;
    }
    h.point_fixed[k] = d->point_fixed ? (d->point_fixed[k] ? 1 : 0) : 0;
  }
  const size_t E = d->n_edges;
  const int K = d->n_poses, P = d->n_points, C = d->n_cams;
  // bulk copies (one array per pool task), then branch-free validation of
  // contiguous edge ranges in parallel (the failing edge is looked up only
  // when a range reports a problem)
  HostPool& pool = HostPool::get();
  // the arrays are sized first (the bulk ones without a zero fill), then
  // filled in pieces of at most 32K edges spread over the pool, so that no
  // single array (the 12-byte observations) is one thread's work
  h.e_type.resize(E);
  h.e_pose.resize(E);
  h.e_point.resize(E);
  h.e_cam.resize(E);
  h.e_obs.resize(3 * E);
  h.e_info.resize(E);
  h.e_delta.resize(E);
  h.e_robust.resize(E);
  h.e_level.resize(E);
  constexpr size_t kPieceEdges = 32768;
  const int npieces = (int)((E + kPieceEdges - 1) / kPieceEdges);
  pool.run(npieces * 9, [&](int t) {
    const int task = t % 9;
    const size_t b = (size_t)(t / 9) * kPieceEdges, e = std::min(E, b + kPieceEdges), n = e - b;
    switch (task) {
      case 0: std::memcpy(h.e_type.data() + b, d->edge_type + b, n); break;
      case 1: std::memcpy(h.e_pose.data() + b, d->edge_pose + b, n * sizeof(int32_t)); break;
      case 2: std::memcpy(h.e_point.data() + b, d->edge_point + b, n * sizeof(int32_t)); break;
      case 3: std::memcpy(h.e_cam.data() + b, d->edge_cam + b, n * sizeof(int32_t)); break;
      case 4: std::memcpy(h.e_obs.data() + 3 * b, d->edge_obs + 3 * b, 3 * n * sizeof(float)); break;
      case 5:
        if (d->edge_info) std::memcpy(h.e_info.data() + b, d->edge_info + b, n * sizeof(float));
        else std::fill(h.e_info.begin() + b, h.e_info.begin() + e, 1.f);
        break;
      case 6:
        if (d->edge_delta) std::memcpy(h.e_delta.data() + b, d->edge_delta + b, n * sizeof(float));
        else std::fill(h.e_delta.begin() + b, h.e_delta.begin() + e, 0.f);
        break;
      case 7:
        if (d->edge_robust)
          for (size_t i = b; i < e; ++i) h.e_robust[i] = d->edge_robust[i] ? 1 : 0;
        else
          std::fill(h.e_robust.begin() + b, h.e_robust.begin() + e, (uint8_t)1);
        break;
      default:
        if (d->edge_level) std::memcpy(h.e_level.data() + b, d->edge_level + b, n);
        else std::fill(h.e_level.begin() + b, h.e_level.begin() + e, (uint8_t)0);
        break;
    }
  });
  // one simple loop per array, branch-free, so that each vectorises
  auto nonfinite_any = [](const float* v, size_t n) {
    const uint32_t* b = reinterpret_cast<const uint32_t*>(v);
    uint32_t bad = 0;
    for (size_t i = 0; i < n; ++i) bad |= (uint32_t)((b[i] & 0x7f800000u) == 0x7f800000u);
    return bad;
  };
  auto out_of_range = [](const int32_t* v, size_t n, int lim) {
    const uint32_t* u = reinterpret_cast<const uint32_t*>(v);
    uint32_t bad = 0;
    for (size_t i = 0; i < n; ++i) bad |= (uint32_t)(u[i] >= (uint32_t)lim);
    return bad;
  };
  constexpr int kParts = 16;
  unsigned flags[kParts][4] = {};
  size_t nun[kParts] = {};
  const size_t per = (E + kParts - 1) / kParts;
  pool.run(E >= 4096 ? kParts : 1, [&](int q) {
    const size_t b = (E >= 4096) ? (size_t)q * per : 0, e = (E >= 4096) ? std::min(E, b + per) : E;
    if (b >= e) return;
    const size_t n = e - b;
    unsigned bt = 0;
    size_t nu = 0;
    for (size_t i = b; i < e; ++i) {
      const uint8_t t = h.e_type[i];
      bt |= (unsigned)(t > MCBA_EDGE_UNARY);
      nu += (size_t)(t == MCBA_EDGE_UNARY);
    }
    flags[q][0] = bt;
    flags[q][1] = out_of_range(h.e_pose.data() + b, n, K) | out_of_range(h.e_point.data() + b, n, P) |
                  out_of_range(h.e_cam.data() + b, n, C);
    flags[q][2] = nonfinite_any(h.e_obs.data() + 3 * b, 3 * n);
    flags[q][3] = nonfinite_any(h.e_info.data() + b, n) | nonfinite_any(h.e_delta.data() + b, n);
    nun[q] = nu;
  });
  unsigned bad_type = 0, bad_index = 0, bad_obs = 0, bad_w = 0;
  size_t n_unary = 0;
  for (int q = 0; q < kParts; ++q) {
    bad_type |= flags[q][0];
    bad_index |= flags[q][1];
    bad_obs |= flags[q][2];
    bad_w |= flags[q][3];
    n_unary += nun[q];
  }
  if (bad_type) return fail(p, MCBA_ERR_INVALID, "unknown edge type");
  if (bad_index) return fail(p, MCBA_ERR_INVALID, "edge index out of range");
  if (bad_obs) return fail(p, MCBA_ERR_NONFINITE, "non-finite observation");
  if (bad_w) return fail(p, MCBA_ERR_NONFINITE, "non-finite information or Huber threshold");
  h.u_Xw.clear();
  if (n_unary) {
    h.u_Xw.reserve(3 * n_unary);
    for (size_t i = 0; i < E; ++i)
      if (h.e_type[i] == MCBA_EDGE_UNARY) {
        for (int a = 0; a < 3; ++a) h.u_Xw.push_back(d->point_Xw[3 * (size_t)h.e_point[i] + a]);
        h.e_point[i] = -1;
      }
  }
  return MCBA_OK;
}

int mcba_edge_count(const mcba_problem* p, int32_t* n) {
  if (!p || !n) return MCBA_ERR_INVALID;
  *n = (int32_t)p->hp.n_edges();
  return MCBA_OK;
}

int mcba_vertex_count(const mcba_problem* p, int32_t* nk, int32_t* np) {
  if (!p) return MCBA_ERR_INVALID;
  if (nk) *nk = (int32_t)p->hp.poses.size();
  if (np) *np = (int32_t)p->hp.point_fixed.size();
  return MCBA_OK;
}

namespace {
void fill_stats(mcba_stats* st, const SolveResult& res, const Structure* s, int status) {
  if (!st) return;
  st->iterations = res.iterations;
  st->trials = res.trials;
  st->status = status;
  st->initial_chi2 = res.initial_chi2;
  st->final_chi2 = res.final_chi2;
  st->lambda = res.lambda;
  if (s) {
    st->n_active_edges = s->E;
    st->n_free_poses = s->Kf;
    st->n_free_points = s->Lf;
  }
  st->edges_linearized = (int64_t)st->n_active_edges * (res.iterations > 0 ? res.iterations : 0);
  st->ms_total = res.ms_total;
  st->ms_linearize = res.ms_linearize;
  for (int i = 0; i < MCBA_NUM_PHASES; ++i) {
    st->ms_phase[i] = res.ms_phase[i];
    st->n_phase[i] = res.n_phase[i];
  }
  st->kernel_launches = res.launches;
  st->h2d_bytes = res.h2d;
  st->d2h_bytes = res.d2h;
}

RunOptions run_options(const mcba_problem* p, int iterations) {
  RunOptions o;
  o.iterations = iterations;
  o.tau = p->opt.tau;
  o.max_trials = p->opt.max_trials;
  o.use_graph = p->opt.use_graph != 0;
  o.profile = p->opt.profile != 0;
  return o;
}
}  // namespace

namespace {
// initializeOptimization + buildStructure and the upload of the problem:
// on the device by default, on the host when mcba_options.host_structure is
// set.  Returns MCBA_ERR_EMPTY when no vertex is left to optimise.
int compile_and_upload(mcba_problem* p, SolveResult& res, std::string& e) {
  StructureSizes z{};
  int r;
  if (p->opt.host_structure) {
    if (!compile_structure(p->hp, p->st)) return MCBA_ERR_EMPTY;
    r = solver_upload(p->solver, p->hp, &p->st, &z, res, &e);
  } else {
    r = solver_upload(p->solver, p->hp, nullptr, &z, res, &e);
    p->st = Structure();
    p->st.K = z.K;
    p->st.P = z.P;
    p->st.U = z.U;
    p->st.Kf = z.Kf;
    p->st.Lf = z.Lf;
    p->st.E = z.E;
    p->st.Ec = z.Ec;
  }
  return r;
}
}  // namespace

int mcba_optimize(mcba_problem* p, int32_t iterations, mcba_stats* st) {
  if (!p || iterations < 0) return fail(p, MCBA_ERR_INVALID, "bad argument");
  if (st) std::memset(st, 0, sizeof(*st));
  int r = ensure_solver(p);
  if (r) return r;
  const auto t0 = std::chrono::steady_clock::now();
  SolveResult res;
  std::string e;
  r = compile_and_upload(p, res, e);
  if (st) {
    st->n_active_edges = p->st.E;
    st->n_free_poses = p->st.Kf;
    st->n_free_points = p->st.Lf;
  }
  if (r == MCBA_ERR_EMPTY) {
    p->log.clear();
    p->prepared = false;
    if (st) {
      st->iterations = -1;
      st->status = MCBA_ERR_EMPTY;
    }
    return fail(p, MCBA_ERR_EMPTY, "0 vertices to optimize");
  }
  const double ms_prep =
      std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (!r) r = solver_run(p->solver, run_options(p, iterations), false, res, &e);
  if (!r) r = solver_download(p->solver, p->hp, res, &e);
  p->prepared = false;
  p->log = res.log;
  p->hpp = res.hpp;
  p->hpp_kf = p->st.Kf;
  fill_stats(st, res, &p->st, r);
  if (st) st->ms_host_prepare = ms_prep;
  if (r) return fail(p, r, e);
  return MCBA_OK;
}

int mcba_prepare(mcba_problem* p) {
  if (!p) return MCBA_ERR_INVALID;
  int r = ensure_solver(p);
  if (r) return r;
  SolveResult res;
  std::string e;
  r = compile_and_upload(p, res, e);
  if (r == MCBA_ERR_EMPTY) return fail(p, MCBA_ERR_EMPTY, "0 vertices to optimize");
  if (r) return fail(p, r, e);
  p->prepared = true;
  return MCBA_OK;
}

int mcba_batch_prepare(mcba_problem* const* problems, int32_t n) {
  if (n < 0 || (n > 0 && !problems)) return MCBA_ERR_INVALID;
  for (int32_t i = 0; i < n; ++i) {
    if (!problems[i]) return MCBA_ERR_INVALID;
    const int r = mcba_prepare(problems[i]);
    if (r) return r;
  }
  return MCBA_OK;
}

int mcba_batch_solve(mcba_problem* const* problems, int32_t n, int32_t iterations, mcba_stats* stats,
                     double* ms_device) {
  if (n < 0 || iterations < 0 || (n > 0 && !problems)) return MCBA_ERR_INVALID;
  if (n == 0) return MCBA_OK;
  std::vector<Solver*> ss(n);
  for (int32_t i = 0; i < n; ++i) {
    mcba_problem* p = problems[i];
    if (!p) return MCBA_ERR_INVALID;
    if (stats) std::memset(&stats[i], 0, sizeof(mcba_stats));
    if (!p->prepared || !solver_has_upload(p->solver)) return fail(p, MCBA_ERR_INVALID, "mcba_batch_prepare first");
    ss[i] = p->solver;
  }
  std::vector<SolveResult> res(n);
  std::string e;
  const int r = solver_run_batch(ss.data(), n, run_options(problems[0], iterations), res.data(), ms_device, &e);
  for (int32_t i = 0; i < n; ++i) {
    mcba_problem* p = problems[i];
    p->log = res[i].log;
    p->hpp = res[i].hpp;
    p->hpp_kf = p->st.Kf;
    if (stats) fill_stats(&stats[i], res[i], &p->st, r);
  }
  if (r) return fail(problems[0], r, e);
  return MCBA_OK;
}

int mcba_batch_solve_persistent(mcba_problem* const* problems, int32_t n, int32_t iterations, mcba_stats* stats,
                                double* ms_device, int32_t* cluster_ctas) {
  if (n < 0 || iterations < 0 || (n > 0 && !problems)) return MCBA_ERR_INVALID;
  if (n == 0) return MCBA_OK;
  std::vector<Solver*> ss(n);
  for (int32_t i = 0; i < n; ++i) {
    mcba_problem* p = problems[i];
    if (!p) return MCBA_ERR_INVALID;
    if (stats) std::memset(&stats[i], 0, sizeof(mcba_stats));
    if (!p->prepared || !solver_has_upload(p->solver)) return fail(p, MCBA_ERR_INVALID, "mcba_batch_prepare first");
    ss[i] = p->solver;
  }
  std::vector<SolveResult> res(n);
  std::string e;
  int ctas = cluster_ctas ? *cluster_ctas : 0;
  const int r = solver_run_batch_persistent(ss.data(), n, run_options(problems[0], iterations), res.data(), ms_device,
                                            &ctas, &e);
  if (cluster_ctas) *cluster_ctas = ctas;
  for (int32_t i = 0; i < n; ++i) {
    mcba_problem* p = problems[i];
    p->log = res[i].log;
    p->hpp = res[i].hpp;
    p->hpp_kf = p->st.Kf;
    if (stats) fill_stats(&stats[i], res[i], &p->st, r);
  }
  if (r) return fail(problems[0], r, e);
  return MCBA_OK;
}

int mcba_solve_prepared(mcba_problem* p, int32_t iterations, mcba_stats* st) {
  if (!p || iterations < 0) return fail(p, MCBA_ERR_INVALID, "bad argument");
  if (st) std::memset(st, 0, sizeof(*st));
  if (!p->prepared || !solver_has_upload(p->solver)) return fail(p, MCBA_ERR_INVALID, "mcba_prepare first");
  SolveResult res;
  std::string e;
  const int r = solver_run(p->solver, run_options(p, iterations), true, res, &e);
  p->log = res.log;
  p->hpp = res.hpp;
  p->hpp_kf = p->st.Kf;
  fill_stats(st, res, &p->st, r);
  if (r) return fail(p, r, e);
  return MCBA_OK;
}

int mcba_fetch_state(mcba_problem* p) {
  if (!p) return MCBA_ERR_INVALID;
  if (!p->prepared || !solver_has_upload(p->solver)) return fail(p, MCBA_ERR_INVALID, "nothing on the device");
  SolveResult res;
  std::string e;
  const int r = solver_download(p->solver, p->hp, res, &e);
  if (r) return fail(p, r, e);
  return MCBA_OK;
}

int mcba_trial_log_get(const mcba_problem* p, mcba_trial_log* out, int32_t cap, int32_t* n) {
  if (!p || cap < 0 || (cap > 0 && !out)) return MCBA_ERR_INVALID;
  const int32_t m = (int32_t)std::min<size_t>(p->log.size(), (size_t)cap);
  if (m) std::memcpy(out, p->log.data(), m * sizeof(mcba_trial_log));
  if (n) *n = (int32_t)p->log.size();
  return MCBA_OK;
}

int mcba_edge_chi2(mcba_problem* p, double* chi2) {
  if (!p || !chi2) return fail(p, MCBA_ERR_INVALID, "null argument");
  if (p->hp.n_edges() == 0) return MCBA_OK;
  int r = ensure_solver(p);
  if (r) return r;
  std::vector<double> v;
  std::string e;
  p->prepared = false;
  r = solver_edge_chi2(p->solver, p->hp, v, &e);
  if (r) return fail(p, r, e);
  std::memcpy(chi2, v.data(), v.size() * sizeof(double));
  return MCBA_OK;
}

int mcba_set_edge_levels(mcba_problem* p, const uint8_t* lv) {
  if (!p || (!lv && p->hp.n_edges())) return fail(p, MCBA_ERR_INVALID, "null argument");
  for (size_t i = 0; i < p->hp.n_edges(); ++i) p->hp.e_level[i] = lv[i];
  return MCBA_OK;
}

int mcba_get_edge_levels(const mcba_problem* p, uint8_t* lv) {
  if (!p || (!lv && p->hp.n_edges())) return MCBA_ERR_INVALID;
  for (size_t i = 0; i < p->hp.n_edges(); ++i) lv[i] = p->hp.e_level[i];
  return MCBA_OK;
}

int mcba_set_edge_robust(mcba_problem* p, const uint8_t* rb) {
  if (!p || (!rb && p->hp.n_edges())) return fail(p, MCBA_ERR_INVALID, "null argument");
  for (size_t i = 0; i < p->hp.n_edges(); ++i) p->hp.e_robust[i] = rb[i] ? 1 : 0;
  return MCBA_OK;
}

int mcba_get_keyframe(const mcba_problem* p, int32_t id, float T[16]) {
  if (!p || !T || id < 0 || id >= (int)p->hp.poses.size()) return MCBA_ERR_INVALID;
  qt_to_mat44f(p->hp.poses[id], T);
  return MCBA_OK;
}

int mcba_get_keyframe_qt(const mcba_problem* p, int32_t id, double qt[7]) {
  if (!p || !qt || id < 0 || id >= (int)p->hp.poses.size()) return MCBA_ERR_INVALID;
  for (int i = 0; i < 4; ++i) qt[i] = p->hp.poses[id].q[i];
  for (int i = 0; i < 3; ++i) qt[4 + i] = p->hp.poses[id].t[i];
  return MCBA_OK;
}

int mcba_get_mappoint(const mcba_problem* p, int32_t id, float X[3]) {
  if (!p || !X || id < 0 || id >= (int)p->hp.point_fixed.size()) return MCBA_ERR_INVALID;
  for (int d = 0; d < 3; ++d) X[d] = (float)p->hp.points[3 * (size_t)id + d];
  return MCBA_OK;
}

int mcba_get_state(const mcba_problem* p, double* qt, double* X) {
  if (!p) return MCBA_ERR_INVALID;
  if (qt)
    for (size_t k = 0; k < p->hp.poses.size(); ++k) {
      for (int i = 0; i < 4; ++i) qt[7 * k + i] = p->hp.poses[k].q[i];
      for (int i = 0; i < 3; ++i) qt[7 * k + 4 + i] = p->hp.poses[k].t[i];
    }
  if (X && !p->hp.points.empty()) std::memcpy(X, p->hp.points.data(), p->hp.points.size() * sizeof(double));
  return MCBA_OK;
}

int mcba_set_state(mcba_problem* p, const double* qt, const double* X) {
  if (!p) return MCBA_ERR_INVALID;
  HostProblem& h = p->hp;
  if (qt) {
    for (size_t k = 0; k < h.poses.size(); ++k)
      for (int i = 0; i < 7; ++i)
        if (!std::isfinite(qt[7 * k + i])) return fail(p, MCBA_ERR_NONFINITE, "non-finite pose");
    for (size_t k = 0; k < h.poses.size(); ++k) {
      const double* a = qt + 7 * k;
      double x = a[0], y = a[1], z = a[2], w = a[3];
      if (w < 0) {
        x = -x;
        y = -y;
        z = -z;
        w = -w;
      }
      const double n = std::sqrt(x * x + y * y + z * z + w * w);
      if (!(n > 0)) return fail(p, MCBA_ERR_INVALID, "zero quaternion");
      QT& T = h.poses[k];
      T.q[0] = x / n;
      T.q[1] = y / n;
      T.q[2] = z / n;
      T.q[3] = w / n;
      for (int i = 0; i < 3; ++i) T.t[i] = a[4 + i];
    }
  }
  if (X) {
    for (size_t i = 0; i < h.points.size(); ++i)
      if (!std::isfinite(X[i])) return fail(p, MCBA_ERR_NONFINITE, "non-finite point");
    std::memcpy(h.points.data(), X, h.points.size() * sizeof(double));
  }
  return MCBA_OK;
}

// SparseBlockMatrix::writeOctave(upperTriangle = true)
// (core/sparse_block_matrix.hpp:555, reached from block_solver.hpp:590-593):
// "# name: H / # type: sparse matrix / # nnz / # rows / # columns" then
// 1-based "row col value" triplets in column-major order.
int mcba_dump_hessian(mcba_problem* p, const char* path) {
  if (!p || !path) return fail(p, MCBA_ERR_INVALID, "null argument");
  const int Kf = p->hpp_kf;
  const int n = 6 * Kf;
  std::vector<int> rr, cc;
  std::vector<double> vv;
  for (int c = 0; c < n; ++c)
    for (int r = 0; r <= c; ++r) {
      if (r / 6 != c / 6 || p->hpp.empty()) continue;
      const int b = r / 6;
      rr.push_back(r + 1);
      cc.push_back(c + 1);
      vv.push_back(p->hpp[36 * (size_t)b + 6 * (r % 6) + (c % 6)]);
    }
  FILE* f = std::fopen(path, "w");
  if (!f) return fail(p, MCBA_ERR_INVALID, std::string("cannot open ") + path);
  std::fprintf(f, "# name: H\n# type: sparse matrix\n# nnz: %zu\n# rows: %d\n# columns: %d\n", vv.size(), n, n);
  for (size_t i = 0; i < vv.size(); ++i) std::fprintf(f, "%d %d %.17g\n", rr[i], cc[i], vv[i]);
  std::fclose(f);
  return MCBA_OK;
}

// src/PoseEstimation.cpp:76-129
int mcba_pose_optimization(mcba_problem* p, int32_t rounds, int32_t iters, float thr, int32_t drop_round,
                           int32_t* inliers, int32_t* written) {
  if (!p || rounds < 0 || iters < 0) return fail(p, MCBA_ERR_INVALID, "bad argument");
  HostProblem& h = p->hp;
  const int nInitial = (int)h.n_edges();
  if (inliers) *inliers = 0;
  if (written) *written = 0;
  if (nInitial < 3) return MCBA_OK;
  int nBad = 0;
  std::vector<double> chi2;
  for (int it = 0; it < rounds; ++it) {
    int r = mcba_optimize(p, iters, nullptr);
    if (r != MCBA_OK && r != MCBA_ERR_EMPTY && r != MCBA_ERR_NOT_PD) return r;
    chi2.resize(h.n_edges());
    r = mcba_edge_chi2(p, chi2.data());
    if (r) return r;
    nBad = 0;
    for (int i = 0; i < nInitial; ++i) {
      if (h.e_level[i] == 1) continue;
      if ((float)chi2[i] >= thr) {
        h.e_level[i] = 1;
        nBad++;
      }
      if (it == drop_round) h.e_robust[i] = 0;
    }
    if (nInitial - nBad < 10) break;
  }
  if (inliers) *inliers = nInitial - nBad;
  if (written) *written = (nInitial - nBad < 10) ? 0 : 1;
  return MCBA_OK;
}

// include/PoseEstimation.hpp:104-118 with src/PoseEstimation.cpp:132-151
int mcba_local_window(mcba_problem* p, const mcba_map_desc* m, int32_t cur, int32_t hop, uint8_t* kf_role,
                      int32_t* pose_kf, int32_t* point_mp, uint8_t* point_fixed, mcba_window_info* info) {
  if (!p || !m) return fail(p, MCBA_ERR_INVALID, "null argument");
  const int K = m->n_keyframes, P = m->n_points;
  if (K <= 0 || K >= (1 << 24) || P < 0 || hop < 1 || cur < 0 || cur >= K || m->n_levels <= 0)
    return fail(p, MCBA_ERR_INVALID, "bad window arguments");
  if (!m->kf_id || !m->kf_Tcw || !m->obs_begin || !m->mp_kf_begin || !m->ess_begin || !m->inv_sigma2_left ||
      !m->inv_sigma2_wide || (P && !m->mp_Xw))
    return fail(p, MCBA_ERR_INVALID, "null map table");
  const int32_t O = m->obs_begin[K], B = m->mp_kf_begin[P], A = m->ess_begin[K];
  if (O >= (1 << 29)) return fail(p, MCBA_ERR_TOO_LARGE, "more than 2^29 observations");
  if (m->obs_begin[0] != 0 || m->mp_kf_begin[0] != 0 || m->ess_begin[0] != 0 || O < 0 || B < 0 || A < 0 ||
      m->obs_begin[cur] < 0 || m->obs_begin[cur + 1] < m->obs_begin[cur] || m->obs_begin[cur + 1] > O)
    return fail(p, MCBA_ERR_INVALID, "bad CSR table bounds");
  if ((O && (!m->obs_point || !m->obs_object || !m->obs_uv || !m->obs_ur || !m->obs_octave)) ||
      (B && !m->mp_kf) || (A && !m->ess_adj))
    return fail(p, MCBA_ERR_INVALID, "null map table");
  for (int k = 0; k < K; ++k)
    if (m->kf_id[k] < 0 || m->kf_id[k] >= (int64_t(1) << 39)) return fail(p, MCBA_ERR_INVALID, "keyframe id out of range");
  // monotone offsets: the ranges are disjoint, so the window has at most 2 O
  // edges (a keyframe is an anchor, a window member or both)
  for (int k = 0; k < K; ++k)
    if (m->obs_begin[k + 1] < m->obs_begin[k] || m->ess_begin[k + 1] < m->ess_begin[k])
      return fail(p, MCBA_ERR_INVALID, "CSR offsets not monotone");
  for (int i = 0; i < P; ++i)
    if (m->mp_kf_begin[i + 1] < m->mp_kf_begin[i]) return fail(p, MCBA_ERR_INVALID, "CSR offsets not monotone");
  WindowHost w;
  std::string e;
  const int r = window_assemble(p->opt.device, m, cur, hop, w, &e);
  if (r) return fail(p, r, e);
  // the problem: camera 0 LEFT (T_cam_body = I, stereo bf), camera 1 WIDE
  const float I4[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
  float camK[8], camT[32];
  const float camB[2] = {m->bf, 0.f};
  std::memcpy(camK, m->K_left, sizeof(float) * 4);
  std::memcpy(camK + 4, m->K_wide, sizeof(float) * 4);
  std::memcpy(camT, I4, sizeof(I4));
  std::memcpy(camT + 16, m->T_wide_body, sizeof(float) * 16);
  const int NPo = (int)w.pose_kf.size(), NPt = (int)w.point_mp.size(), E = (int)w.e_type.size();
  std::vector<float> T((size_t)NPo * 16), X((size_t)NPt * 3);
  for (int i = 0; i < NPo; ++i) std::memcpy(&T[16 * (size_t)i], m->kf_Tcw + 16 * (size_t)w.pose_kf[i], 64);
  for (int i = 0; i < NPt; ++i) std::memcpy(&X[3 * (size_t)i], m->mp_Xw + 3 * (size_t)w.point_mp[i], 12);
  mcba_problem_desc d{};
  d.n_cams = 2;
  d.cam_K = camK;
  d.cam_bf = camB;
  d.cam_Tcb = camT;
  d.n_poses = NPo;
  d.pose_Tcw = T.data();
  d.pose_fixed = w.pose_fixed.data();
  d.n_points = NPt;
  d.point_Xw = X.data();
  d.point_fixed = w.point_fixed.data();
  d.n_edges = E;
  d.edge_type = w.e_type.data();
  d.edge_pose = w.e_pose.data();
  d.edge_point = w.e_point.data();
  d.edge_cam = w.e_cam.data();
  d.edge_obs = w.e_obs.data();
  d.edge_info = w.e_info.data();
  d.edge_delta = w.e_delta.data();
  const int rl = mcba_load(p, &d);
  if (rl) return rl;
  if (kf_role) std::memcpy(kf_role, w.kf_role.data(), (size_t)K);
  if (pose_kf && NPo) std::memcpy(pose_kf, w.pose_kf.data(), sizeof(int32_t) * NPo);
  if (point_mp && NPt) std::memcpy(point_mp, w.point_mp.data(), sizeof(int32_t) * NPt);
  if (point_fixed && NPt) std::memcpy(point_fixed, w.point_fixed.data(), (size_t)NPt);
  if (info) {
    info->n_local = w.n_local;
    info->n_anchor = w.n_anchor;
    info->n_poses = NPo;
    info->n_points = NPt;
    info->n_fixed_points = w.n_fixed_points;
    info->n_edges = E;
  }
  return MCBA_OK;
}

int mcba_local_ba(mcba_problem* p, int32_t iters, float thr, int32_t* success, int32_t* written) {
  if (!p || iters < 0) return fail(p, MCBA_ERR_INVALID, "bad argument");
  int r = mcba_optimize(p, iters, nullptr);
  if (r != MCBA_OK && r != MCBA_ERR_EMPTY && r != MCBA_ERR_NOT_PD) return r;
  HostProblem& h = p->hp;
  std::vector<double> chi2(h.n_edges());
  if (!chi2.empty()) {
    r = mcba_edge_chi2(p, chi2.data());
    if (r) return r;
  }
  for (size_t i = 0; i < h.n_edges(); ++i) {
    if (h.e_level[i] == 1) continue;
    if ((float)chi2[i] >= thr) h.e_level[i] = 1;
  }
  const int init_cnt = (int)h.n_edges();
  if (success) *success = init_cnt;
  if (written) *written = init_cnt > 10 ? 1 : 0;
  return MCBA_OK;
}

}  // extern "C"
