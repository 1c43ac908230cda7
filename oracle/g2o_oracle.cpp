// g2o_oracle.cpp -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
//
// CPU restatement of MCVSLAM's bundle-adjustment path (BAoptimizer on top of
// g2o's Levenberg-Marquardt with a 6/3 block Schur solver).  Used only by the
// test suite, the smoke check and the benchmark's CPU legs, as the checker and
// the timed CPU baseline.  Parity is UNPINNED: the reference has no golden
// vectors and cannot be built here (no Eigen3), so this file follows the
// reference source line by line instead (citations below are paths inside the
// reference project; g2o files are under ThirdParty/g2o/g2o/).
//
// Eigen operations the reference relies on are restated from the published
// formulas: Hamilton quaternion product, quaternion-vector rotation
// v + 2w(q x v) + 2 q x (q x v), rotation matrix -> quaternion (Shoemake's
// trace/largest-diagonal method), 3x3 inverse by the adjugate, and a dense
// LL^T factorisation restricted to the skyline of the reduced camera matrix
// in place of Eigen's SimplicialLLT with AMD ordering (same factor up to
// round-off; the pattern is fixed per optimize call just like the symbolic
// analysis in solvers/eigen/linear_solver_eigen.h:130-160).

#include "g2o_oracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------- SE3Quat --
// types/slam3d/se3quat.h:36-296 (quaternion + translation, w >= 0, unit norm)
struct Quat {
  double x, y, z, w;
};
struct SE3 {
  Quat r;
  double t[3];
};

inline Quat qmul(const Quat& a, const Quat& b) {
  Quat o;
  o.w = a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z;
  o.x = a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y;
  o.y = a.w * b.y + a.y * b.w + a.z * b.x - a.x * b.z;
  o.z = a.w * b.z + a.z * b.w + a.x * b.y - a.y * b.x;
  return o;
}

// se3quat.h:280-285 normalizeRotation: flip to w >= 0, then unit norm.
inline void se3_normalize(SE3& T) {
  if (T.r.w < 0) {
    T.r.x = -T.r.x;
    T.r.y = -T.r.y;
    T.r.z = -T.r.z;
    T.r.w = -T.r.w;
  }
  const double n = std::sqrt(T.r.x * T.r.x + T.r.y * T.r.y + T.r.z * T.r.z + T.r.w * T.r.w);
  T.r.x /= n;
  T.r.y /= n;
  T.r.z /= n;
  T.r.w /= n;
}

// Rotation of a vector by a unit quaternion: v + w*uv + q x uv, uv = 2 q x v.
inline void qrot(const Quat& q, const double v[3], double o[3]) {
  double uv[3] = {q.y * v[2] - q.z * v[1], q.z * v[0] - q.x * v[2], q.x * v[1] - q.y * v[0]};
  uv[0] += uv[0];
  uv[1] += uv[1];
  uv[2] += uv[2];
  const double c[3] = {q.y * uv[2] - q.z * uv[1], q.z * uv[0] - q.x * uv[2], q.x * uv[1] - q.y * uv[0]};
  o[0] = v[0] + q.w * uv[0] + c[0];
  o[1] = v[1] + q.w * uv[1] + c[1];
  o[2] = v[2] + q.w * uv[2] + c[2];
}

// se3quat.h:212-215 map(xyz) = r*xyz + t
inline void se3_map(const SE3& T, const double X[3], double o[3]) {
  qrot(T.r, X, o);
  o[0] += T.t[0];
  o[1] += T.t[1];
  o[2] += T.t[2];
}

// se3quat.h:99-105 operator*: t += r*t2, r *= r2, normalize.
inline SE3 se3_compose(const SE3& a, const SE3& b) {
  SE3 o = a;
  double rt[3];
  qrot(a.r, b.t, rt);
  o.t[0] += rt[0];
  o.t[1] += rt[1];
  o.t[2] += rt[2];
  o.r = qmul(a.r, b.r);
  se3_normalize(o);
  return o;
}

// Unit quaternion -> row-major rotation matrix (standard 2x/2y/2z form).
inline void q2R(const Quat& q, double R[9]) {
  const double tx = 2 * q.x, ty = 2 * q.y, tz = 2 * q.z;
  const double twx = tx * q.w, twy = ty * q.w, twz = tz * q.w;
  const double txx = tx * q.x, txy = ty * q.x, txz = tz * q.x;
  const double tyy = ty * q.y, tyz = tz * q.y, tzz = tz * q.z;
  R[0] = 1 - (tyy + tzz);
  R[1] = txy - twz;
  R[2] = txz + twy;
  R[3] = txy + twz;
  R[4] = 1 - (txx + tzz);
  R[5] = tyz - twx;
  R[6] = txz - twy;
  R[7] = tyz + twx;
  R[8] = 1 - (txx + tyy);
}

// Rotation matrix -> quaternion, Shoemake's method (positive trace branch,
// otherwise the largest diagonal element picks the leading component).
inline Quat R2q(const double R[9]) {
  Quat q;
  double tr = R[0] + R[4] + R[8];
  if (tr > 0) {
    double s = std::sqrt(tr + 1.0);
    q.w = 0.5 * s;
    s = 0.5 / s;
    q.x = (R[7] - R[5]) * s;
    q.y = (R[2] - R[6]) * s;
    q.z = (R[3] - R[1]) * s;
  } else {
    int i = 0;
    if (R[4] > R[0]) i = 1;
    if (R[8] > R[i * 3 + i]) i = 2;
    const int j = (i + 1) % 3, k = (j + 1) % 3;
    double s = std::sqrt(R[i * 3 + i] - R[j * 3 + j] - R[k * 3 + k] + 1.0);
    double v[3];
    v[i] = 0.5 * s;
    s = 0.5 / s;
    q.w = (R[k * 3 + j] - R[j * 3 + k]) * s;
    v[j] = (R[j * 3 + i] + R[i * 3 + j]) * s;
    v[k] = (R[k * 3 + i] + R[i * 3 + k]) * s;
    q.x = v[0];
    q.y = v[1];
    q.z = v[2];
  }
  return q;
}

// se3quat.h:53-55 SE3Quat(R, t)
inline SE3 se3_from_Rt(const double R[9], const double t[3]) {
  SE3 T;
  T.r = R2q(R);
  T.t[0] = t[0];
  T.t[1] = t[1];
  T.t[2] = t[2];
  se3_normalize(T);
  return T;
}

// src/Converter.cc:31-39 toSE3Quat(float 4x4)
inline SE3 se3_from_mat44f(const float* M) {
  const double R[9] = {M[0], M[1], M[2], M[4], M[5], M[6], M[8], M[9], M[10]};
  const double t[3] = {M[3], M[7], M[11]};
  return se3_from_Rt(R, t);
}

// src/Converter.cc:41-52 toCvMat(SE3Quat): homogeneous matrix cast to float.
inline void se3_to_mat44f(const SE3& T, float* M) {
  double R[9];
  q2R(T.r, R);
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) M[i * 4 + j] = (float)R[i * 3 + j];
    M[i * 4 + 3] = (float)T.t[i];
  }
  M[12] = 0.f;
  M[13] = 0.f;
  M[14] = 0.f;
  M[15] = 1.f;
}

inline void skew(const double w[3], double S[9]) {
  S[0] = 0;
  S[1] = -w[2];
  S[2] = w[1];
  S[3] = w[2];
  S[4] = 0;
  S[5] = -w[0];
  S[6] = -w[1];
  S[7] = w[0];
  S[8] = 0;
}

inline void mat3mul(const double A[9], const double B[9], double C[9]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) C[i * 3 + j] = A[i * 3] * B[j] + A[i * 3 + 1] * B[3 + j] + A[i * 3 + 2] * B[6 + j];
}

// se3quat.h:218-257 SE3Quat::exp (series below theta = 1e-5, Rodrigues above)
inline SE3 se3_exp(const double u[6]) {
  const double omega[3] = {u[0], u[1], u[2]};
  const double ups[3] = {u[3], u[4], u[5]};
  const double theta = std::sqrt(omega[0] * omega[0] + omega[1] * omega[1] + omega[2] * omega[2]);
  double O[9], O2[9], R[9], V[9];
  skew(omega, O);
  mat3mul(O, O, O2);
  double a, b;  // R = I + a O + b O2 ; V = I + vb O + vc O2
  double vb, vc;
  if (theta < 0.00001) {
    a = 1.0;
    b = 0.5;
    vb = 0.5;
    vc = 1.0 / 6.0;
  } else {
    a = std::sin(theta) / theta;
    b = (1 - std::cos(theta)) / (theta * theta);
    vb = b;
    vc = (theta - std::sin(theta)) / std::pow(theta, 3);
  }
  for (int i = 0; i < 9; ++i) {
    const double I = (i % 4 == 0) ? 1.0 : 0.0;
    R[i] = I + a * O[i] + b * O2[i];
    V[i] = I + vb * O[i] + vc * O2[i];
  }
  double t[3];
  for (int i = 0; i < 3; ++i) t[i] = V[i * 3] * ups[0] + V[i * 3 + 1] * ups[1] + V[i * 3 + 2] * ups[2];
  return se3_from_Rt(R, t);
}

// ------------------------------------------------------------ camera/edge --
struct Cam {
  double fx, fy, cx, cy;  // float parameters promoted (BaseCamera.hpp:43)
  double bf;
  SE3 Tcb;
};

// modules/camera/Pinhole.cpp:55-60 project(Eigen::Vector3d)
inline void project(const Cam& c, const double P[3], double o[2]) {
  o[0] = c.fx * P[0] / P[2] + c.cx;
  o[1] = c.fy * P[1] / P[2] + c.cy;
}

// modules/camera/Pinhole.cpp:105-116 projectJac(Eigen::Vector3d)
inline void projectJac(const Cam& c, const double P[3], double J[6]) {
  J[0] = c.fx / P[2];
  J[1] = 0.0;
  J[2] = -c.fx * P[0] / (P[2] * P[2]);
  J[3] = 0.0;
  J[4] = c.fy / P[2];
  J[5] = -c.fy * P[1] / (P[2] * P[2]);
}

struct Edge {
  int type, pose, point, cam, dim;
  double obs[3];
  double info, delta;
  bool robust;
  int level;
  double Pw[3];
  double err[3];
  double Jl[3][3];
  double Jp[3][6];
};

struct Graph {
  std::vector<Cam> cams;
  std::vector<SE3> poses;
  std::vector<uint8_t> pose_fixed;
  std::vector<double> points;  // 3 per point
  std::vector<uint8_t> point_fixed;
  std::vector<Edge> edges;
};

// robust_kernel_impl.cpp:65-78 RobustKernelHuber::robustify
inline void huber(double e, double delta, double rho[3]) {
  const double dsqr = delta * delta;
  if (e <= dsqr) {
    rho[0] = e;
    rho[1] = 1.;
    rho[2] = 0.;
  } else {
    const double sqrte = std::sqrt(e);
    rho[0] = 2 * sqrte * delta - dsqr;
    rho[1] = delta / sqrte;
    rho[2] = -0.5 * rho[1] / e;
  }
}

// base_edge.h:94-97 chi2 = e' * Omega * e with Omega = invSigma2 * I
inline double edge_chi2(const Edge& e) {
  double s = 0;
  for (int k = 0; k < e.dim; ++k) s += e.err[k] * (e.info * e.err[k]);
  return s;
}

// computeError of the three edge types
//  mono   : include/OptimizeTypes.hpp:80-86  e = z - pi((Tcb * Tbw).map(X))
//  unary  : include/OptimizeTypes.hpp:29-33  same with the constant Pw
//  stereo : include/OptimizeTypes.hpp:127-133,144-154 with float invz and
//           the float product bf*invz of cam_project_uv_u
void compute_error(const Graph& g, Edge& e) {
  const SE3& T = g.poses[e.pose];
  const double* X = (e.type == ORC_EDGE_UNARY) ? e.Pw : &g.points[3 * e.point];
  const Cam& c = g.cams[e.cam];
  if (e.type == ORC_EDGE_STEREO) {
    double Pc[3];
    se3_map(T, X, Pc);
    const float invz = (float)(1.0 / Pc[2]);
    const double u = Pc[0] * (double)invz * c.fx + c.cx;
    const double v = Pc[1] * (double)invz * c.fy + c.cy;
    const float bff = (float)c.bf;
    const double ur = u - (double)(bff * invz);
    e.err[0] = e.obs[0] - u;
    e.err[1] = e.obs[1] - v;
    e.err[2] = e.obs[2] - ur;
  } else {
    const SE3 Tcw = se3_compose(c.Tcb, T);
    double Pc[3], uv[2];
    se3_map(Tcw, X, Pc);
    project(c, Pc, uv);
    e.err[0] = e.obs[0] - uv[0];
    e.err[1] = e.obs[1] - uv[1];
    e.err[2] = 0.0;
  }
}

// linearizeOplus of the three edge types
//  mono   : include/OptimizeTypes.hpp:94-113
//  unary  : include/OptimizeTypes.hpp:40-63
//  stereo : src/OptimizeTypes.cpp:12-58
void linearize(const Graph& g, Edge& e) {
  const SE3& T = g.poses[e.pose];
  const double* X = (e.type == ORC_EDGE_UNARY) ? e.Pw : &g.points[3 * e.point];
  const Cam& c = g.cams[e.cam];
  std::memset(e.Jl, 0, sizeof(e.Jl));
  std::memset(e.Jp, 0, sizeof(e.Jp));
  if (e.type == ORC_EDGE_STEREO) {
    double R[9], P[3];
    q2R(T.r, R);
    se3_map(T, X, P);
    const double x = P[0], y = P[1], z = P[2], z_2 = z * z;
    const double fx = c.fx, fy = c.fy, bf = c.bf;
    for (int j = 0; j < 3; ++j) {
      e.Jl[0][j] = -fx * R[j] / z + fx * x * R[6 + j] / z_2;
      e.Jl[1][j] = -fy * R[3 + j] / z + fy * y * R[6 + j] / z_2;
      e.Jl[2][j] = e.Jl[0][j] - bf * R[6 + j] / z_2;
    }
    e.Jp[0][0] = x * y / z_2 * fx;
    e.Jp[0][1] = -(1 + (x * x / z_2)) * fx;
    e.Jp[0][2] = y / z * fx;
    e.Jp[0][3] = -1. / z * fx;
    e.Jp[0][4] = 0;
    e.Jp[0][5] = x / z_2 * fx;
    e.Jp[1][0] = (1 + y * y / z_2) * fy;
    e.Jp[1][1] = -x * y / z_2 * fy;
    e.Jp[1][2] = -x / z * fy;
    e.Jp[1][3] = 0;
    e.Jp[1][4] = -1. / z * fy;
    e.Jp[1][5] = y / z_2 * fy;
    e.Jp[2][0] = e.Jp[0][0] - bf * y / z_2;
    e.Jp[2][1] = e.Jp[0][1] + bf * x / z_2;
    e.Jp[2][2] = e.Jp[0][2];
    e.Jp[2][3] = e.Jp[0][3];
    e.Jp[2][4] = 0;
    e.Jp[2][5] = e.Jp[0][5] - bf / z_2;
    return;
  }
  double Pb[3], Pc[3], Jpi[6], Rcb[9];
  se3_map(T, X, Pb);
  se3_map(c.Tcb, Pb, Pc);
  projectJac(c, Pc, Jpi);
  q2R(c.Tcb.r, Rcb);
  // M = -Jpi * Rcb (2x3)
  double M[6];
  for (int r = 0; r < 2; ++r)
    for (int j = 0; j < 3; ++j)
      M[r * 3 + j] = -Jpi[r * 3] * Rcb[j] + -Jpi[r * 3 + 1] * Rcb[3 + j] + -Jpi[r * 3 + 2] * Rcb[6 + j];
  // SE3deriv = [ -[Pb]x | I ]
  const double xb = Pb[0], yb = Pb[1], zb = Pb[2];
  const double D[18] = {0., zb, -yb, 1., 0., 0., -zb, 0., xb, 0., 1., 0., yb, -xb, 0., 0., 0., 1.};
  for (int r = 0; r < 2; ++r)
    for (int j = 0; j < 6; ++j) e.Jp[r][j] = M[r * 3] * D[j] + M[r * 3 + 1] * D[6 + j] + M[r * 3 + 2] * D[12 + j];
  if (e.type == ORC_EDGE_MONO) {
    const SE3 Tcw = se3_compose(c.Tcb, T);
    double Rcw[9];
    q2R(Tcw.r, Rcw);
    for (int r = 0; r < 2; ++r)
      for (int j = 0; j < 3; ++j)
        e.Jl[r][j] = -Jpi[r * 3] * Rcw[j] + -Jpi[r * 3 + 1] * Rcw[3 + j] + -Jpi[r * 3 + 2] * Rcw[6 + j];
  }
}

// ----------------------------------------------------------------- solver --
struct TimerS {
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  double s() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

struct HplBlock {
  int pose_idx;    // Hessian pose index (row block)
  double B[18];    // 6x3, row-major
};

class Optimizer {
 public:
  Graph& g;
  int n_threads;
  std::vector<int> active;     // active edge ids, internal-id order
  std::vector<int> pose_idx;   // per pose: Hessian index or -1
  std::vector<int> point_idx;  // per point: landmark index or -1
  std::vector<int> free_poses, free_points;
  int Kf = 0, Lf = 0, n = 0;
  std::vector<double> Hpp, Hll, b, x;
  std::vector<std::vector<int>> col_blocks;  // per landmark: HplBlock ids sorted by pose_idx
  std::vector<HplBlock> hpl;
  std::vector<int> edge_slot;  // per active edge position: hpl block id or -1
  std::vector<int> sky;        // skyline: first nonzero column per row of S
  std::vector<double> S, L, bs, coeff, Dinv;
  std::vector<uint8_t> pose_has_pair;
  // per-vertex edge lists for the threaded accumulation
  std::vector<std::vector<int>> pose_edges, point_edges;
  std::vector<int> pose_only_edges;  // active edges without a free point
  double lambda = -1, ni = 2;
  orc_result* r = nullptr;
  double t_lin = 0;
  int64_t n_lin = 0;

  Optimizer(Graph& g_, int nt) : g(g_), n_threads(nt) {}

  // sparse_optimizer.cpp:201-272 initializeOptimization(level 0) and
  // :168-188 buildIndexMapping: active edges are level-0 edges with at least
  // one free vertex; free poses first, then free points, each in id order.
  bool initialize() {
    active.clear();
    pose_idx.assign(g.poses.size(), -1);
    point_idx.assign(g.points.size() / 3, -1);
    std::vector<uint8_t> pose_act(g.poses.size(), 0), point_act(g.points.size() / 3, 0);
    for (int i = 0; i < (int)g.edges.size(); ++i) {
      const Edge& e = g.edges[i];
      if (e.level != 0) continue;
      const bool pf = g.pose_fixed[e.pose] != 0;
      const bool xf = (e.type == ORC_EDGE_UNARY) ? true : (g.point_fixed[e.point] != 0);
      if (pf && xf) continue;  // allVerticesFixed (sparse_optimizer.cpp:237)
      active.push_back(i);
      pose_act[e.pose] = 1;
      if (e.type != ORC_EDGE_UNARY) point_act[e.point] = 1;
    }
    free_poses.clear();
    free_points.clear();
    for (int k = 0; k < (int)g.poses.size(); ++k)
      if (pose_act[k] && !g.pose_fixed[k]) {
        pose_idx[k] = (int)free_poses.size();
        free_poses.push_back(k);
      }
    for (int k = 0; k < (int)point_idx.size(); ++k)
      if (point_act[k] && !g.point_fixed[k]) {
        point_idx[k] = (int)free_points.size();
        free_points.push_back(k);
      }
    Kf = (int)free_poses.size();
    Lf = (int)free_points.size();
    n = 6 * Kf;
    return (Kf + Lf) > 0;
  }

  // block_solver.hpp:103-256 buildStructure: Hpp/Hll diagonal blocks, one Hpl
  // block per (pose, landmark) pair, Schur pattern from co-observations.
  void build_structure() {
    Hpp.assign((size_t)Kf * 36, 0.0);
    Hll.assign((size_t)Lf * 9, 0.0);
    b.assign((size_t)n + 3 * Lf, 0.0);
    x.assign((size_t)n + 3 * Lf, 0.0);
    col_blocks.assign(Lf, {});
    hpl.clear();
    edge_slot.assign(active.size(), -1);
    pose_edges.assign(Kf, {});
    point_edges.assign(Lf, {});
    pose_only_edges.clear();
    for (size_t a = 0; a < active.size(); ++a) {
      const Edge& e = g.edges[active[a]];
      const int pi = pose_idx[e.pose];
      const int li = (e.type == ORC_EDGE_UNARY) ? -1 : point_idx[e.point];
      if (pi >= 0) pose_edges[pi].push_back((int)a);
      if (li >= 0) point_edges[li].push_back((int)a);
      if (li < 0) pose_only_edges.push_back((int)a);
      if (pi < 0 || li < 0) continue;
      int found = -1;
      for (int bid : col_blocks[li])
        if (hpl[bid].pose_idx == pi) found = bid;
      if (found < 0) {
        HplBlock hb;
        hb.pose_idx = pi;
        std::memset(hb.B, 0, sizeof(hb.B));
        found = (int)hpl.size();
        hpl.push_back(hb);
        col_blocks[li].push_back(found);
      }
      edge_slot[a] = found;
    }
    for (auto& col : col_blocks)
      std::sort(col.begin(), col.end(), [&](int p, int q) { return hpl[p].pose_idx < hpl[q].pose_idx; });
    // skyline of S by pose rows: first co-observing pose index per row
    std::vector<int> firstblk(Kf);
    for (int i = 0; i < Kf; ++i) firstblk[i] = i;
    for (auto& col : col_blocks) {
      if (col.empty()) continue;
      const int lo = hpl[col.front()].pose_idx;
      for (int bid : col) firstblk[hpl[bid].pose_idx] = std::min(firstblk[hpl[bid].pose_idx], lo);
    }
    sky.assign(n, 0);
    for (int i = 0; i < Kf; ++i)
      for (int d = 0; d < 6; ++d) sky[6 * i + d] = 6 * firstblk[i];
    S.assign((size_t)n * n, 0.0);
    L.assign((size_t)n * n, 0.0);
    bs.assign(n, 0.0);
    coeff.assign(n, 0.0);
    Dinv.assign((size_t)Lf * 9, 0.0);
  }

  // sparse_optimizer.cpp:63-90 computeActiveErrors
  void compute_errors() {
    const int na = (int)active.size();
#pragma omp parallel for num_threads(n_threads) if (n_threads > 1 && na > 50)
    for (int k = 0; k < na; ++k) compute_error(g, g.edges[active[k]]);
  }

  // sparse_optimizer.cpp:102-116 activeRobustChi2
  double robust_term(const Edge& e) const {
    if (!e.robust) return edge_chi2(e);
    double rho[3];
    huber(edge_chi2(e), e.delta, rho);
    return rho[0];
  }
  double robust_chi2() const {
    const int na = (int)active.size();
    if (n_threads <= 1 || na < 4096) {
      double chi = 0.0;
      for (int id : active) chi += robust_term(g.edges[id]);
      return chi;
    }
    // static chunks summed in chunk order: deterministic for a thread count
    std::vector<double> part(n_threads, 0.0);
#pragma omp parallel for num_threads(n_threads) schedule(static, 1)
    for (int t = 0; t < n_threads; ++t) {
      const int a0 = (int)((int64_t)na * t / n_threads), a1 = (int)((int64_t)na * (t + 1) / n_threads);
      double c = 0.0;
      for (int a = a0; a < a1; ++a) c += robust_term(g.edges[active[a]]);
      part[t] = c;
    }
    double chi = 0.0;
    for (double c : part) chi += c;
    return chi;
  }

  // Per-edge quadratic-form terms (base_binary_edge.hpp:64-136,
  // base_unary_edge.hpp:51-79) with Omega = info*I and, for the robust
  // branch, W = rho' * Omega (base_edge.h:143-149: no rho'' term).
  struct EdgeTerms {
    double Hll[9], bl[3], Hpp[36], bp[6], Hpl[18];
  };

  void edge_terms(const Edge& e, bool point_free, bool pose_free, EdgeTerms& t) const {
    double w = e.info, s = 1.0;
    if (e.robust) {
      double rho[3];
      huber(edge_chi2(e), e.delta, rho);
      w = rho[1] * e.info;
      s = rho[1];
    }
    double om[3];
    for (int k = 0; k < e.dim; ++k) om[k] = -(e.info * e.err[k]) * s;
    if (point_free) {
      for (int i = 0; i < 3; ++i) {
        double acc = 0;
        for (int k = 0; k < e.dim; ++k) acc += e.Jl[k][i] * om[k];
        t.bl[i] = acc;
        for (int j = 0; j < 3; ++j) {
          double h = 0;
          for (int k = 0; k < e.dim; ++k) h += (e.Jl[k][i] * w) * e.Jl[k][j];
          t.Hll[i * 3 + j] = h;
        }
      }
      if (pose_free)
        for (int i = 0; i < 6; ++i)
          for (int j = 0; j < 3; ++j) {
            double h = 0;
            for (int k = 0; k < e.dim; ++k) h += (e.Jp[k][i] * w) * e.Jl[k][j];
            t.Hpl[i * 3 + j] = h;
          }
    }
    if (pose_free) {
      for (int i = 0; i < 6; ++i) {
        double acc = 0;
        for (int k = 0; k < e.dim; ++k) acc += e.Jp[k][i] * om[k];
        t.bp[i] = acc;
        for (int j = 0; j < 6; ++j) {
          double h = 0;
          for (int k = 0; k < e.dim; ++k) h += (e.Jp[k][i] * w) * e.Jp[k][j];
          t.Hpp[i * 6 + j] = h;
        }
      }
    }
  }

  // block_solver.hpp:463-521 buildSystem
  void build_system() {
    TimerS tm;
    std::fill(Hpp.begin(), Hpp.end(), 0.0);
    std::fill(Hll.begin(), Hll.end(), 0.0);
    std::fill(b.begin(), b.end(), 0.0);
    for (auto& h : hpl) std::memset(h.B, 0, sizeof(h.B));
    const int na = (int)active.size();
    if (n_threads <= 1) {
      EdgeTerms t;
      for (int a = 0; a < na; ++a) {
        Edge& e = g.edges[active[a]];
        linearize(g, e);
        const int pi = pose_idx[e.pose];
        const int li = (e.type == ORC_EDGE_UNARY) ? -1 : point_idx[e.point];
        edge_terms(e, li >= 0, pi >= 0, t);
        if (li >= 0) {
          for (int i = 0; i < 3; ++i) b[n + 3 * li + i] += t.bl[i];
          for (int i = 0; i < 9; ++i) Hll[9 * li + i] += t.Hll[i];
          if (pi >= 0)
            for (int i = 0; i < 18; ++i) hpl[edge_slot[a]].B[i] += t.Hpl[i];
        }
        if (pi >= 0) {
          for (int i = 0; i < 6; ++i) b[6 * pi + i] += t.bp[i];
          for (int i = 0; i < 36; ++i) Hpp[36 * pi + i] += t.Hpp[i];
        }
      }
    } else {
      // threaded variant: the edges of one free point are linearised and
      // accumulated by one thread (point terms and Hpl blocks are private to
      // it); pose terms go to per-thread copies summed in thread order
      // afterwards (g2o's optional OpenMP build locks the vertices instead)
#ifdef _OPENMP
      const int nt = n_threads;
      priv_pose.assign((size_t)nt * Kf * 42, 0.0);
#pragma omp parallel num_threads(nt)
      {
        double* P = &priv_pose[(size_t)omp_get_thread_num() * Kf * 42];
        EdgeTerms t;
        auto pose_terms = [&](int pi) {
          for (int i = 0; i < 6; ++i) P[42 * pi + 36 + i] += t.bp[i];
          for (int i = 0; i < 36; ++i) P[42 * pi + i] += t.Hpp[i];
        };
#pragma omp for schedule(dynamic, 64) nowait
        for (int li = 0; li < Lf; ++li)
          for (int a : point_edges[li]) {
            Edge& e = g.edges[active[a]];
            linearize(g, e);
            const int pi = pose_idx[e.pose];
            edge_terms(e, true, pi >= 0, t);
            for (int i = 0; i < 3; ++i) b[n + 3 * li + i] += t.bl[i];
            for (int i = 0; i < 9; ++i) Hll[9 * li + i] += t.Hll[i];
            if (pi >= 0) {
              for (int i = 0; i < 18; ++i) hpl[edge_slot[a]].B[i] += t.Hpl[i];
              pose_terms(pi);
            }
          }
#pragma omp for schedule(static)
        for (size_t q = 0; q < pose_only_edges.size(); ++q) {
          const int a = pose_only_edges[q];
          Edge& e = g.edges[active[a]];
          linearize(g, e);
          const int pi = pose_idx[e.pose];
          edge_terms(e, false, pi >= 0, t);
          if (pi >= 0) pose_terms(pi);
        }
#pragma omp for schedule(static)
        for (int pi = 0; pi < Kf; ++pi)
          for (int tt = 0; tt < nt; ++tt) {
            const double* Q = &priv_pose[((size_t)tt * Kf + pi) * 42];
            for (int i = 0; i < 36; ++i) Hpp[36 * pi + i] += Q[i];
            for (int i = 0; i < 6; ++i) b[6 * pi + i] += Q[36 + i];
          }
      }
#endif
    }
    t_lin += tm.s();
    n_lin += na;
  }

  // optimization_algorithm_levenberg.cpp:145-157 computeLambdaInit
  double lambda_init() const {
    double m = 0;
    for (int i = 0; i < Kf; ++i)
      for (int j = 0; j < 6; ++j) m = std::max(std::fabs(Hpp[36 * i + 7 * j]), m);
    for (int i = 0; i < Lf; ++i)
      for (int j = 0; j < 3; ++j) m = std::max(std::fabs(Hll[9 * i + 4 * j]), m);
    return 1e-5 * m;
  }

  static bool inv3(const double D[9], double o[9]) {
    const double c00 = D[4] * D[8] - D[5] * D[7];
    const double c01 = D[5] * D[6] - D[3] * D[8];
    const double c02 = D[3] * D[7] - D[4] * D[6];
    const double det = D[0] * c00 + D[1] * c01 + D[2] * c02;
    const double id = 1.0 / det;
    o[0] = c00 * id;
    o[1] = (D[2] * D[7] - D[1] * D[8]) * id;
    o[2] = (D[1] * D[5] - D[2] * D[4]) * id;
    o[3] = c01 * id;
    o[4] = (D[0] * D[8] - D[2] * D[6]) * id;
    o[5] = (D[2] * D[3] - D[0] * D[5]) * id;
    o[6] = c02 * id;
    o[7] = (D[1] * D[6] - D[0] * D[7]) * id;
    o[8] = (D[0] * D[4] - D[1] * D[3]) * id;
    return true;
  }

  // block_solver.hpp:315-447 solve() with the diagonal already damped by
  // setLambda (block_solver.hpp:524-550; lambda is passed in and added here
  // so that H itself is never modified -- restoreDiagonal is then implicit).
  bool solve(double lam) {
    const int NP = n;
    // Hschur = Hpp (upper triangle), coefficients = 0
    std::fill(S.begin(), S.end(), 0.0);
    for (int i = 0; i < Kf; ++i)
      for (int r = 0; r < 6; ++r)
        for (int c = r; c < 6; ++c)
          S[(size_t)(6 * i + r) * NP + 6 * i + c] = Hpp[36 * i + 6 * r + c] + (r == c ? lam : 0.0);
    std::fill(coeff.begin(), coeff.end(), 0.0);
    auto landmark = [&](int li, double* Sacc, double* cacc, bool locked) {
      double D[9];
      for (int i = 0; i < 9; ++i) D[i] = Hll[9 * li + i];
      D[0] += lam;
      D[4] += lam;
      D[8] += lam;
      double* Di = &Dinv[9 * li];
      inv3(D, Di);
      double db[3];
      const double* bl = &b[n + 3 * li];
      for (int i = 0; i < 3; ++i) db[i] = Di[3 * i] * bl[0] + Di[3 * i + 1] * bl[1] + Di[3 * i + 2] * bl[2];
      const auto& col = col_blocks[li];
      for (size_t a = 0; a < col.size(); ++a) {
        const HplBlock& Bi = hpl[col[a]];
        const int i1 = Bi.pose_idx;
        double BD[18];
        for (int r = 0; r < 6; ++r)
          for (int c = 0; c < 3; ++c)
            BD[r * 3 + c] = Bi.B[r * 3] * Di[c] + Bi.B[r * 3 + 1] * Di[3 + c] + Bi.B[r * 3 + 2] * Di[6 + c];
        if (locked) lock_row(i1);
        for (int r = 0; r < 6; ++r)
          cacc[6 * i1 + r] += Bi.B[r * 3] * db[0] + Bi.B[r * 3 + 1] * db[1] + Bi.B[r * 3 + 2] * db[2];
        for (size_t q = a; q < col.size(); ++q) {
          const HplBlock& Bj = hpl[col[q]];
          const int i2 = Bj.pose_idx;
          for (int r = 0; r < 6; ++r)
            for (int c = 0; c < 6; ++c) {
              const double v = BD[r * 3] * Bj.B[c * 3] + BD[r * 3 + 1] * Bj.B[c * 3 + 1] + BD[r * 3 + 2] * Bj.B[c * 3 + 2];
              Sacc[(size_t)(6 * i1 + r) * NP + 6 * i2 + c] -= v;
            }
        }
        if (locked) unlock_row(i1);
      }
    };
    if (n_threads <= 1) {
      for (int li = 0; li < Lf; ++li) landmark(li, S.data(), coeff.data(), false);
    } else if ((size_t)NP * NP * n_threads <= ((size_t)8 << 20)) {
#ifdef _OPENMP
      // Thread-private reduced-camera accumulators summed afterwards.  g2o's
      // optional OpenMP build locks block rows instead (block_solver.hpp:
      // 371-373); with few keyframes that serialises the threads, so the
      // multi-core baseline accumulates privately when the copies are small.
      priv_S.assign((size_t)n_threads * NP * NP, 0.0);
      priv_c.assign((size_t)n_threads * NP, 0.0);
#pragma omp parallel num_threads(n_threads)
      {
        const int t = omp_get_thread_num();
        double* St = &priv_S[(size_t)t * NP * NP];
        double* ct = &priv_c[(size_t)t * NP];
#pragma omp for schedule(dynamic, 16)
        for (int li = 0; li < Lf; ++li) landmark(li, St, ct, false);
#pragma omp for schedule(static)
        for (int row = 0; row < NP; ++row) {
          double* Sr = &S[(size_t)row * NP];
          for (int tt = 0; tt < n_threads; ++tt) {
            const double* Pr = &priv_S[((size_t)tt * NP + row) * NP];
            for (int c = row - row % 6; c < NP; ++c) Sr[c] += Pr[c];
            coeff[row] += priv_c[(size_t)tt * NP + row];
          }
        }
      }
#endif
    } else {
#pragma omp parallel for num_threads(n_threads) schedule(dynamic, 10)
      for (int li = 0; li < Lf; ++li) landmark(li, S.data(), coeff.data(), true);
    }
    for (int i = 0; i < NP; ++i) bs[i] = b[i] - coeff[i];
    // LL^T of the upper triangle (diagonal blocks: upper part only)
    if (!cholesky()) return false;
    // forward / backward substitution
    std::vector<double> y(NP);
    for (int i = 0; i < NP; ++i) {
      double s = bs[i];
      for (int k = sky[i]; k < i; ++k) s -= L[(size_t)i * NP + k] * y[k];
      y[i] = s / L[(size_t)i * NP + i];
    }
    for (int i = NP - 1; i >= 0; --i) {
      double s = y[i];
      for (int k = i + 1; k < NP; ++k)
        if (sky[k] <= i) s -= L[(size_t)k * NP + i] * x[k];
      x[i] = s / L[(size_t)i * NP + i];
    }
    // landmarks: cl = bl - Hpl^T xp ; xl = Dinv cl
#pragma omp parallel for num_threads(n_threads) schedule(static) if (n_threads > 1)
    for (int li = 0; li < Lf; ++li) {
      double cl[3] = {b[n + 3 * li], b[n + 3 * li + 1], b[n + 3 * li + 2]};
      for (int bid : col_blocks[li]) {
        const HplBlock& B = hpl[bid];
        for (int c = 0; c < 3; ++c)
          for (int r = 0; r < 6; ++r) cl[c] += B.B[r * 3 + c] * (-x[6 * B.pose_idx + r]);
      }
      const double* Di = &Dinv[9 * li];
      for (int i = 0; i < 3; ++i) x[n + 3 * li + i] = Di[3 * i] * cl[0] + Di[3 * i + 1] * cl[1] + Di[3 * i + 2] * cl[2];
    }
    return true;
  }

  // Column-by-column LL^T on the skyline of S (S stored as its upper
  // triangle and read as S[j][i] for i > j; L row-major lower).  Each column
  // j needs only columns < j, so the rows below the pivot are independent.
  // Fails like SimplicialLLT on a non-positive pivot (a NaN pivot passes).
  bool cholesky() {
    const int NP = n;
    for (int j = 0; j < NP; ++j) {
      const double* Lj = &L[(size_t)j * NP];
      double d = S[(size_t)j * NP + j];
      for (int k = sky[j]; k < j; ++k) d -= Lj[k] * Lj[k];
      if (d <= 0.0) return false;
      const double ljj = std::sqrt(d);
      L[(size_t)j * NP + j] = ljj;
      if (n_threads > 1 && NP - j > 64) {
#pragma omp parallel for num_threads(n_threads) schedule(static)
        for (int i = j + 1; i < NP; ++i) col_entry(i, j, ljj);
      } else {
        for (int i = j + 1; i < NP; ++i) col_entry(i, j, ljj);
      }
    }
    return true;
  }
  inline void col_entry(int i, int j, double ljj) {
    if (sky[i] > j) return;
    const int NP = n;
    const int k0 = std::max(sky[i], sky[j]);
    double s = S[(size_t)j * NP + i];
    const double* Li = &L[(size_t)i * NP];
    const double* Lj = &L[(size_t)j * NP];
    for (int k = k0; k < j; ++k) s -= Li[k] * Lj[k];
    L[(size_t)i * NP + j] = s / ljj;
  }

  std::vector<double> priv_S, priv_c;  // thread-private Schur accumulators
  std::vector<double> priv_pose;  // per-thread pose terms of the threaded linearisation

  // Per-row locks for the threaded Schur loop (block_solver.hpp:371-373).
#ifdef _OPENMP
  std::vector<omp_lock_t> locks;
  void init_locks() {
    if (n_threads > 1 && (int)locks.size() != Kf) {
      for (auto& l : locks) omp_destroy_lock(&l);
      locks.resize(Kf);
      for (auto& l : locks) omp_init_lock(&l);
    }
  }
  void lock_row(int i) {
    if (n_threads > 1) omp_set_lock(&locks[i]);
  }
  void unlock_row(int i) {
    if (n_threads > 1) omp_unset_lock(&locks[i]);
  }
  ~Optimizer() {
    for (auto& l : locks) omp_destroy_lock(&l);
  }
#else
  void init_locks() {}
  void lock_row(int) {}
  void unlock_row(int) {}
#endif

  // sparse_optimizer.cpp:433-446 update -> VertexSE3Expmap::oplusImpl
  // (types_six_dof_expmap.h:98-101) and VertexSBAPointXYZ::oplusImpl
  // (types_sba.h:146-150)
  void update() {
    for (int i = 0; i < Kf; ++i) {
      SE3& T = g.poses[free_poses[i]];
      T = se3_compose(se3_exp(&x[6 * i]), T);
    }
    for (int i = 0; i < Lf; ++i) {
      double* X = &g.points[3 * free_points[i]];
      X[0] += x[n + 3 * i];
      X[1] += x[n + 3 * i + 1];
      X[2] += x[n + 3 * i + 2];
    }
  }

  // optimization_algorithm_levenberg.cpp:159-165 computeScale
  double compute_scale(double lam) const {
    double s = 0;
    for (size_t j = 0; j < x.size(); ++j) s += x[j] * (lam * x[j] + b[j]);
    return s;
  }

  void log_trial(int it, int q, double chi0, double chi1, double lam, double sc, double rho, bool acc, bool ok) {
    if (!r || !r->log) {
      if (r) r->n_log++;
      return;
    }
    if (r->n_log < r->log_cap) {
      orc_trial_log& L_ = r->log[r->n_log];
      L_.iteration = it;
      L_.trial = q;
      L_.chi_before = chi0;
      L_.chi_after = chi1;
      L_.lambda = lam;
      L_.scale = sc;
      L_.rho = rho;
      L_.accepted = acc ? 1 : 0;
      L_.solve_ok = ok ? 1 : 0;
    }
    r->n_log++;
  }

  // sparse_optimizer.cpp:366-431 optimize + optimization_algorithm_levenberg.cpp:56-143 solve
  int optimize(int iterations) {
    if (!initialize()) return -1;
    init_locks();
    int done = 0;
    bool ok = true;
    for (int it = 0; it < iterations && ok; ++it) {
      if (it == 0) build_structure();
      compute_errors();
      double currentChi = robust_chi2();
      build_system();
      if (it == 0) {
        lambda = lambda_init();
        ni = 2;
      }
      double rho = 0;
      int qmax = 0;
      std::vector<SE3> bak_p(Kf);
      std::vector<double> bak_x(3 * (size_t)Lf);
      do {
        for (int i = 0; i < Kf; ++i) bak_p[i] = g.poses[free_poses[i]];
        for (int i = 0; i < Lf; ++i)
          for (int d = 0; d < 3; ++d) bak_x[3 * i + d] = g.points[3 * free_points[i] + d];
        const double lam = lambda;
        const bool ok2 = solve(lam);
        update();
        compute_errors();
        double tempChi = robust_chi2();
        if (!ok2) tempChi = std::numeric_limits<double>::max();
        rho = currentChi - tempChi;
        double scale = compute_scale(lam);
        scale += 1e-3;
        rho /= scale;
        const bool acc = (rho > 0 && std::isfinite(tempChi));
        log_trial(it, qmax, currentChi, tempChi, lam, scale, rho, acc, ok2);
        if (acc) {
          double alpha = 1. - std::pow((2 * rho - 1), 3);
          alpha = std::min(alpha, 2. / 3.);
          const double sf = std::max(1. / 3., alpha);
          lambda *= sf;
          ni = 2;
          currentChi = tempChi;
        } else {
          lambda *= ni;
          ni *= 2;
          for (int i = 0; i < Kf; ++i) g.poses[free_poses[i]] = bak_p[i];
          for (int i = 0; i < Lf; ++i)
            for (int d = 0; d < 3; ++d) g.points[3 * free_points[i] + d] = bak_x[3 * i + d];
          if (!std::isfinite(lambda)) break;
        }
        qmax++;
      } while (rho < 0 && qmax < 10);
      ++done;
      if (qmax == 10 || rho == 0 || !std::isfinite(lambda)) ok = false;
    }
    return done;
  }
};

Graph load(const orc_problem* p) {
  Graph g;
  g.cams.resize(p->n_cams);
  for (int c = 0; c < p->n_cams; ++c) {
    Cam& k = g.cams[c];
    k.fx = p->cam_K[4 * c];
    k.fy = p->cam_K[4 * c + 1];
    k.cx = p->cam_K[4 * c + 2];
    k.cy = p->cam_K[4 * c + 3];
    k.bf = p->cam_bf ? (double)p->cam_bf[c] : 0.0;
    k.Tcb = se3_from_mat44f(&p->cam_Tcb[16 * c]);
  }
  g.poses.resize(p->n_poses);
  g.pose_fixed.resize(p->n_poses);
  for (int k = 0; k < p->n_poses; ++k) {
    g.poses[k] = se3_from_mat44f(&p->pose_Tcw[16 * k]);
    g.pose_fixed[k] = p->pose_fixed ? p->pose_fixed[k] : 0;
  }
  g.points.resize(3 * (size_t)p->n_points);
  g.point_fixed.resize(p->n_points);
  for (int k = 0; k < p->n_points; ++k) {
    for (int d = 0; d < 3; ++d) g.points[3 * k + d] = p->point_Xw[3 * k + d];
    g.point_fixed[k] = p->point_fixed ? p->point_fixed[k] : 0;
  }
  g.edges.resize(p->n_edges);
  for (int i = 0; i < p->n_edges; ++i) {
    Edge& e = g.edges[i];
    e.type = p->edge_type[i];
    e.pose = p->edge_pose[i];
    e.point = p->edge_point[i];
    e.cam = p->edge_cam[i];
    e.dim = (e.type == ORC_EDGE_STEREO) ? 3 : 2;
    for (int d = 0; d < 3; ++d) e.obs[d] = p->edge_obs[3 * i + d];
    e.info = p->edge_info ? (double)p->edge_info[i] : 1.0;
    e.delta = p->edge_delta ? (double)p->edge_delta[i] : 0.0;
    e.robust = p->edge_robust ? (p->edge_robust[i] != 0) : true;
    e.level = p->edge_level ? p->edge_level[i] : 0;
    for (int d = 0; d < 3; ++d) e.Pw[d] = p->point_Xw[3 * e.point + d];
    std::memset(e.err, 0, sizeof(e.err));
  }
  return g;
}

void se3_to_qt(const SE3& T, double* qt) {
  qt[0] = T.r.x;
  qt[1] = T.r.y;
  qt[2] = T.r.z;
  qt[3] = T.r.w;
  qt[4] = T.t[0];
  qt[5] = T.t[1];
  qt[6] = T.t[2];
}
SE3 qt_to_se3(const double* qt) {
  SE3 T;
  T.r = {qt[0], qt[1], qt[2], qt[3]};
  T.t[0] = qt[4];
  T.t[1] = qt[5];
  T.t[2] = qt[6];
  return T;
}

// Final read-back: estimates, per-edge chi2 from a fresh computeError, and
// activeRobustChi2 over the active set.
void write_result(Optimizer& opt, orc_result* r) {
  if (!r) return;
  Graph& g = opt.g;
  for (size_t k = 0; k < g.poses.size(); ++k) {
    if (r->pose_qt) se3_to_qt(g.poses[k], &r->pose_qt[7 * k]);
    if (r->pose_Tcw) se3_to_mat44f(g.poses[k], &r->pose_Tcw[16 * k]);
  }
  if (r->point_X)
    for (size_t k = 0; k < g.points.size(); ++k) r->point_X[k] = g.points[k];
  for (auto& e : g.edges) compute_error(g, e);
  if (r->edge_chi2)
    for (size_t i = 0; i < g.edges.size(); ++i) r->edge_chi2[i] = edge_chi2(g.edges[i]);
  if (r->edge_level)
    for (size_t i = 0; i < g.edges.size(); ++i) r->edge_level[i] = (uint8_t)g.edges[i].level;
  r->n_active_edges = (int32_t)opt.active.size();
  r->final_chi2 = opt.robust_chi2();
  r->seconds_linearize = opt.t_lin;
  r->edges_linearized = opt.n_lin;
}

}  // namespace

extern "C" {

int orc_optimize(const orc_problem* p, int iterations, int n_threads, orc_result* r) {
  TimerS tm;
  Graph g = load(p);
  Optimizer opt(g, n_threads);
  if (r) r->n_log = 0;
  opt.r = r;
  const int ret = opt.optimize(iterations);
  if (r) {
    r->iterations_done = ret;
    write_result(opt, r);
    r->seconds_total = tm.s();
  }
  return ret;
}

// src/PoseEstimation.cpp:48-130
int orc_pose_optimization(const orc_problem* p, int rounds, int iters, float chi2_thr,
                          int drop_robust_round, int n_threads, orc_result* r, int* pose_written) {
  TimerS tm;
  Graph g = load(p);
  Optimizer opt(g, n_threads);
  if (r) r->n_log = 0;
  opt.r = r;
  const int nInitial = (int)g.edges.size();
  if (pose_written) *pose_written = 0;
  if (nInitial < 3) {
    if (r) write_result(opt, r);
    return 0;
  }
  int nBad = 0;
  for (int it = 0; it < rounds; ++it) {
    opt.optimize(iters);
    nBad = 0;
    for (auto& e : g.edges) {
      if (e.level == 1) continue;
      compute_error(g, e);
      const float chi2 = (float)edge_chi2(e);
      if (chi2 >= chi2_thr) {
        e.level = 1;
        nBad++;
      }
      if (it == drop_robust_round) e.robust = false;
    }
    if (nInitial - nBad < 10) break;
  }
  if (pose_written) *pose_written = (nInitial - nBad < 10) ? 0 : 1;
  if (r) {
    write_result(opt, r);
    r->seconds_total = tm.s();
  }
  return nInitial - nBad;
}

// include/PoseEstimation.hpp:104-118 with the chi2 callback of
// src/PoseEstimation.cpp:132-151 (nBad is never incremented: the raw
// callback is passed to filter, include/PoseEstimation.hpp:110-113)
int orc_local_ba(const orc_problem* p, int iterations, float chi2_thr, int n_threads, orc_result* r,
                 int* written) {
  TimerS tm;
  Graph g = load(p);
  Optimizer opt(g, n_threads);
  if (r) r->n_log = 0;
  opt.r = r;
  const int ret = opt.optimize(iterations);
  const int init_cnt = (int)g.edges.size();
  for (auto& e : g.edges) {
    if (e.level == 1) continue;
    compute_error(g, e);
    const float chi2 = (float)edge_chi2(e);
    if (chi2 >= chi2_thr) e.level = 1;
  }
  if (written) *written = init_cnt > 10 ? 1 : 0;
  if (r) {
    r->iterations_done = ret;
    write_result(opt, r);
    r->seconds_total = tm.s();
  }
  return init_cnt;
}

int orc_linearize_edges(const orc_problem* p, double* err, double* J_point, double* J_pose) {
  Graph g = load(p);
  for (size_t i = 0; i < g.edges.size(); ++i) {
    Edge& e = g.edges[i];
    compute_error(g, e);
    linearize(g, e);
    for (int k = 0; k < 3; ++k) {
      if (err) err[3 * i + k] = e.err[k];
      for (int j = 0; j < 3; ++j)
        if (J_point) J_point[9 * i + 3 * k + j] = e.Jl[k][j];
      for (int j = 0; j < 6; ++j)
        if (J_pose) J_pose[18 * i + 6 * k + j] = e.Jp[k][j];
    }
  }
  return (int)g.edges.size();
}

int orc_normal_equations(const orc_problem* p, double lambda, double* H, double* bout, double* x_schur, int cap) {
  Graph g = load(p);
  Optimizer opt(g, 1);
  if (!opt.initialize()) return 0;
  opt.build_structure();
  opt.compute_errors();
  opt.build_system();
  const int N = opt.n + 3 * opt.Lf;
  if (N > cap) return -N;
  if (H) {
    std::fill(H, H + (size_t)N * N, 0.0);
    for (int i = 0; i < opt.Kf; ++i)
      for (int r = 0; r < 6; ++r)
        for (int c = 0; c < 6; ++c) H[(size_t)(6 * i + r) * N + 6 * i + c] = opt.Hpp[36 * i + 6 * r + c];
    for (int l = 0; l < opt.Lf; ++l) {
      const int o = opt.n + 3 * l;
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) H[(size_t)(o + r) * N + o + c] = opt.Hll[9 * l + 3 * r + c];
      for (int bid : opt.col_blocks[l]) {
        const HplBlock& B = opt.hpl[bid];
        for (int r = 0; r < 6; ++r)
          for (int c = 0; c < 3; ++c) {
            H[(size_t)(6 * B.pose_idx + r) * N + o + c] = B.B[r * 3 + c];
            H[(size_t)(o + c) * N + 6 * B.pose_idx + r] = B.B[r * 3 + c];
          }
      }
    }
    for (int i = 0; i < N; ++i) H[(size_t)i * N + i] += lambda;
  }
  if (bout)
    for (int i = 0; i < N; ++i) bout[i] = opt.b[i];
  if (x_schur) {
    const bool ok = opt.solve(lambda);
    for (int i = 0; i < N; ++i) x_schur[i] = ok ? opt.x[i] : NAN;
  }
  return N;
}

void orc_se3_exp(const double u[6], double qt[7]) { se3_to_qt(se3_exp(u), qt); }
void orc_mat44f_to_qt(const float T[16], double qt[7]) { se3_to_qt(se3_from_mat44f(T), qt); }
void orc_qt_to_mat44f(const double qt[7], float T[16]) { se3_to_mat44f(qt_to_se3(qt), T); }
void orc_huber(double e2, double delta, double rho[3]) { huber(e2, delta, rho); }
void orc_compose(const double a[7], const double b[7], double o[7]) {
  se3_to_qt(se3_compose(qt_to_se3(a), qt_to_se3(b)), o);
}
void orc_map(const double qt[7], const double X[3], double o[3]) { se3_map(qt_to_se3(qt), X, o); }

}  // extern "C"
