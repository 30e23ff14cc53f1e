// ORACLE — test infrastructure only.
//
// FP64 restatement of mind-fcl's OBB BVH-vs-BVH boolean collision
// (OrientedNodeBVHSolver::MeshIntersect with penetration off): the OBB overlap
// test, the triangle-triangle separating-axis test, and the traversal order.
// meshIntersect traverses a given flattened FP32 tree (the one the GPU
// library builds); buildRefTree / meshIntersectRef restate the reference's
// own FP64 OBBRSS tree and traverse it exactly as the reference does, so that
// the order of reported contacts, and with it the contacts a capped request
// keeps, follow the reference's.
#pragma once

#include <cmath>
#include <cstdint>
#include <limits>
#include <utility>
#include <vector>

namespace orc {

// Flattened OBB node: axis is row-major 3x3 whose COLUMNS are the box axes
// (the reference's OBB::axis, math/bv/OBB.h), To its center, extent its half
// sizes; child >= 0: internal with children child and child + 1 (the
// reference's BVNodeBase::leftChild / rightChild); child < 0: leaf holding
// triangle -(child + 1).
struct MeshNode {
  float axis[9];
  float center[3];
  float extent[3];
  int32_t child;
};
static_assert(sizeof(MeshNode) == 64, "node layout");

struct Mat3 {
  double m[9];
  double operator()(int r, int c) const { return m[3 * r + c]; }
};

inline double d3dot(const double* a, const double* b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }

// obbDisjoint, math/bv/OBB-inl.h:319-436 (B relative rotation, T relative
// translation in box 1's axes, a / b extents; |B| gets a 1e-6 slack).
inline bool obbDisjoint(const Mat3& B, const double T[3], const double a[3], const double b[3]) {
  const double reps = 1e-6;
  double Bf[9];
  for (int i = 0; i < 9; ++i) Bf[i] = std::abs(B.m[i]) + reps;
  auto row = [&](int r, const double* v) { return (Bf[3 * r] * v[0] + Bf[3 * r + 1] * v[1]) + Bf[3 * r + 2] * v[2]; };
  auto col = [&](int c, const double* v) { return (Bf[c] * v[0] + Bf[3 + c] * v[1]) + Bf[6 + c] * v[2]; };
  auto bcol_dot = [&](int c, const double* v) { return (B.m[c] * v[0] + B.m[3 + c] * v[1]) + B.m[6 + c] * v[2]; };
  double t, s;
  t = std::abs(T[0]);
  if (t > (a[0] + row(0, b))) return true;
  s = bcol_dot(0, T);
  t = std::abs(s);
  if (t > (b[0] + col(0, a))) return true;
  t = std::abs(T[1]);
  if (t > (a[1] + row(1, b))) return true;
  t = std::abs(T[2]);
  if (t > (a[2] + row(2, b))) return true;
  s = bcol_dot(1, T);
  t = std::abs(s);
  if (t > (b[1] + col(1, a))) return true;
  s = bcol_dot(2, T);
  t = std::abs(s);
  if (t > (b[2] + col(2, a))) return true;
  auto Bm = [&](int r, int c) { return B.m[3 * r + c]; };
  auto F = [&](int r, int c) { return Bf[3 * r + c]; };
  s = T[2] * Bm(1, 0) - T[1] * Bm(2, 0);
  if (std::abs(s) > (a[1] * F(2, 0) + a[2] * F(1, 0) + b[1] * F(0, 2) + b[2] * F(0, 1))) return true;
  s = T[2] * Bm(1, 1) - T[1] * Bm(2, 1);
  if (std::abs(s) > (a[1] * F(2, 1) + a[2] * F(1, 1) + b[0] * F(0, 2) + b[2] * F(0, 0))) return true;
  s = T[2] * Bm(1, 2) - T[1] * Bm(2, 2);
  if (std::abs(s) > (a[1] * F(2, 2) + a[2] * F(1, 2) + b[0] * F(0, 1) + b[1] * F(0, 0))) return true;
  s = T[0] * Bm(2, 0) - T[2] * Bm(0, 0);
  if (std::abs(s) > (a[0] * F(2, 0) + a[2] * F(0, 0) + b[1] * F(1, 2) + b[2] * F(1, 1))) return true;
  s = T[0] * Bm(2, 1) - T[2] * Bm(0, 1);
  if (std::abs(s) > (a[0] * F(2, 1) + a[2] * F(0, 1) + b[0] * F(1, 2) + b[2] * F(1, 0))) return true;
  s = T[0] * Bm(2, 2) - T[2] * Bm(0, 2);
  if (std::abs(s) > (a[0] * F(2, 2) + a[2] * F(0, 2) + b[0] * F(1, 1) + b[1] * F(1, 0))) return true;
  s = T[1] * Bm(0, 0) - T[0] * Bm(1, 0);
  if (std::abs(s) > (a[0] * F(1, 0) + a[1] * F(0, 0) + b[1] * F(2, 2) + b[2] * F(2, 1))) return true;
  s = T[1] * Bm(0, 1) - T[0] * Bm(1, 1);
  if (std::abs(s) > (a[0] * F(1, 1) + a[1] * F(0, 1) + b[0] * F(2, 2) + b[2] * F(2, 0))) return true;
  s = T[1] * Bm(0, 2) - T[0] * Bm(1, 2);
  if (std::abs(s) > (a[0] * F(1, 2) + a[1] * F(0, 2) + b[0] * F(2, 1) + b[1] * F(2, 0))) return true;
  return false;
}

// overlap(R0, T0, OBB b1, OBB b2), math/bv/OBB-inl.h:305-316: b2 posed by
// (R0, T0) in b1's mesh frame.
inline bool obbOverlap(const Mat3& R0, const double T0[3], const MeshNode& b1, const MeshNode& b2) {
  double A1[9], A2[9];
  for (int i = 0; i < 9; ++i) { A1[i] = b1.axis[i]; A2[i] = b2.axis[i]; }
  double R0b2[9];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c)
      R0b2[3 * r + c] = (R0.m[3 * r] * A2[c] + R0.m[3 * r + 1] * A2[3 + c]) + R0.m[3 * r + 2] * A2[6 + c];
  Mat3 R;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c)
      R.m[3 * r + c] = (A1[r] * R0b2[c] + A1[3 + r] * R0b2[3 + c]) + A1[6 + r] * R0b2[6 + c];
  double Tt[3];
  for (int r = 0; r < 3; ++r)
    Tt[r] = (((R0.m[3 * r] * b2.center[0] + R0.m[3 * r + 1] * b2.center[1]) + R0.m[3 * r + 2] * b2.center[2]) +
             T0[r]) -
            (double)b1.center[r];
  double T[3];
  for (int c = 0; c < 3; ++c) T[c] = (Tt[0] * A1[c] + Tt[1] * A1[3 + c]) + Tt[2] * A1[6 + c];
  const double a[3] = {b1.extent[0], b1.extent[1], b1.extent[2]};
  const double b[3] = {b2.extent[0], b2.extent[1], b2.extent[2]};
  return !obbDisjoint(R, T, a, b);
}

struct P3 {
  double x, y, z;
};
inline P3 sub(P3 a, P3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline P3 crs(P3 a, P3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double dt(P3 a, P3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }

// project6, narrowphase/detail/traversal/collision/intersect-inl.h:1082-1102
inline bool project6(P3 ax, P3 p1, P3 p2, P3 p3, P3 q1, P3 q2, P3 q3) {
  const double P1 = dt(ax, p1), P2 = dt(ax, p2), P3v = dt(ax, p3);
  const double Q1 = dt(ax, q1), Q2 = dt(ax, q2), Q3 = dt(ax, q3);
  const double mn1 = std::min(P1, std::min(P2, P3v));
  const double mx2 = std::max(Q1, std::max(Q2, Q3));
  if (mn1 > mx2) return false;
  const double mx1 = std::max(P1, std::max(P2, P3v));
  const double mn2 = std::min(Q1, std::min(Q2, Q3));
  if (mn2 > mx1) return false;
  return true;
}

// intersect_Triangle (boolean), intersect-inl.h:593-613 and 723-795: Q
// transformed by (R, T), then the 17-axis separating-axis test relative to P1.
inline bool intersectTriangle(P3 P1, P3 P2, P3 P3_, P3 Q1, P3 Q2, P3 Q3, const Mat3& R, const double T[3]) {
  auto xf = [&](P3 q) {
    return P3{((R.m[0] * q.x + R.m[1] * q.y) + R.m[2] * q.z) + T[0], ((R.m[3] * q.x + R.m[4] * q.y) + R.m[5] * q.z) + T[1],
              ((R.m[6] * q.x + R.m[7] * q.y) + R.m[8] * q.z) + T[2]};
  };
  const P3 Qa = xf(Q1), Qb = xf(Q2), Qc = xf(Q3);
  const P3 p1 = sub(P1, P1), p2 = sub(P2, P1), p3 = sub(P3_, P1);
  const P3 q1 = sub(Qa, P1), q2 = sub(Qb, P1), q3 = sub(Qc, P1);
  const P3 e1 = sub(p2, p1), e2 = sub(p3, p2), e3 = sub(p1, p3);
  const P3 f1 = sub(q2, q1), f2 = sub(q3, q2), f3 = sub(q1, q3);
  const P3 n1 = crs(e1, e2), m1 = crs(f1, f2);
  const P3 axes[17] = {n1, m1, crs(e1, f1), crs(e1, f2), crs(e1, f3), crs(e2, f1), crs(e2, f2), crs(e2, f3),
                       crs(e3, f1), crs(e3, f2), crs(e3, f3), crs(e1, n1), crs(e2, n1), crs(e3, n1), crs(f1, m1),
                       crs(f2, m1), crs(f3, m1)};
  for (const P3& ax : axes)
    if (!project6(ax, p1, p2, p3, q1, q2, q3)) return false;
  return true;
}

// OrientedNodeBVHSolver::MeshIntersect, bvh_solver-inl.h:74-164, boolean
// contacts (b1, b2) until max_contacts (CollisionResult::addContact +
// terminationConditionSatisfied).  (R, T): mesh b's pose in mesh a's frame
// (relativeTransform, math/geometry-inl.h:409-433).
inline void meshIntersect(const MeshNode* na, const float* tri_a, const MeshNode* nb, const float* tri_b,
                          const Mat3& R, const double T[3], size_t max_contacts,
                          std::vector<std::pair<int, int>>& contacts) {
  contacts.clear();
  if (max_contacts == 0) return;
  auto vtx = [](const float* tris, int t, int k) {
    const float* p = tris + 12 * (size_t)t + 4 * k;
    return P3{p[0], p[1], p[2]};
  };
  auto size2 = [](const MeshNode& n) {
    return ((double)n.extent[0] * n.extent[0] + (double)n.extent[1] * n.extent[1]) + (double)n.extent[2] * n.extent[2];
  };
  std::vector<std::pair<int, int>> stack;
  stack.emplace_back(0, 0);
  while (!stack.empty()) {
    const std::pair<int, int> task = stack.back();
    stack.pop_back();
    const MeshNode& a = na[task.first];
    const MeshNode& b = nb[task.second];
    if (!obbOverlap(R, T, a, b)) continue;
    const bool la = a.child < 0, lb = b.child < 0;
    if (la && lb) {
      const int ta = -(a.child + 1), tb = -(b.child + 1);
      if (intersectTriangle(vtx(tri_a, ta, 0), vtx(tri_a, ta, 1), vtx(tri_a, ta, 2), vtx(tri_b, tb, 0),
                            vtx(tri_b, tb, 1), vtx(tri_b, tb, 2), R, T)) {
        contacts.emplace_back(ta, tb);
        if (contacts.size() >= max_contacts) return;
      }
      continue;
    }
    const bool go_a = lb || (!la && size2(a) > size2(b));
    if (go_a) {
      stack.emplace_back(a.child, task.second);
      stack.emplace_back(a.child + 1, task.second);
    } else {
      stack.emplace_back(task.first, b.child);
      stack.emplace_back(task.first, b.child + 1);
    }
  }
}

// ------------------------------------------------ the reference's OBBRSS tree --
//
// FP64 restatement of BVHModel<OBBRSS<double>>::endModel on a triangle mesh
// (geometry/bvh/BVH_model-inl.h:403-440 buildTreeIterativeImpl, :450-570
// iterativeBuildTree) with the default mean splitter: each node's OBB is fitted
// by FitImpl<S, OBBRSS<S>> (geometry/bvh/detail/BV_fitter-inl.h:323-345:
// getCovariance, eigen_old, axisFromEigen, getExtentAndCenter), the split
// vector is the OBB's first axis (BV_splitter-inl.h:449-454), the split value
// the mean of the triangle centroids projected on it (computeSplitValue_mean,
// :464-506), a triangle goes right when its centroid projects above it
// (ApplyImpl<OBBRSS>, :411-415), an empty side falls back to half / half, and
// the children take the next two node slots (left first) with the left
// subtree built first.  Only the OBB half of OBBRSS is kept: the traversal's
// overlap test and the split read only the OBB (OBBRSS-inl.h:114-116, 132-137).
struct RefNode {
  double axis[9];  // row-major; columns are the box axes (OBB::axis)
  double To[3];
  double extent[3];
  double size;     // extent.squaredNorm() (OBB::size, OBB-inl.h:153-156)
  int first_child, first_primitive, num_primitives;
};

// geometry-inl.h:712-767 (triangles only)
inline void refCovariance(const double* V, const int32_t* T, const uint32_t* idx, int n, double M[9]) {
  double S1[3] = {0, 0, 0};
  double S2[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  int n_points = 0;
  for (int i = 0; i < n; ++i) {
    const int32_t* t = T + 3 * (size_t)idx[i];
    const double* p1 = V + 3 * (size_t)t[0];
    const double* p2 = V + 3 * (size_t)t[1];
    const double* p3 = V + 3 * (size_t)t[2];
    for (int k = 0; k < 3; ++k) S1[k] += (p1[k] + p2[k]) + p3[k];
    S2[0][0] += (p1[0] * p1[0] + p2[0] * p2[0] + p3[0] * p3[0]);
    S2[1][1] += (p1[1] * p1[1] + p2[1] * p2[1] + p3[1] * p3[1]);
    S2[2][2] += (p1[2] * p1[2] + p2[2] * p2[2] + p3[2] * p3[2]);
    S2[0][1] += (p1[0] * p1[1] + p2[0] * p2[1] + p3[0] * p3[1]);
    S2[0][2] += (p1[0] * p1[2] + p2[0] * p2[2] + p3[0] * p3[2]);
    S2[1][2] += (p1[1] * p1[2] + p2[1] * p2[2] + p3[1] * p3[2]);
    n_points += 3;
  }
  M[0] = S2[0][0] - S1[0] * S1[0] / n_points;
  M[4] = S2[1][1] - S1[1] * S1[1] / n_points;
  M[8] = S2[2][2] - S1[2] * S1[2] / n_points;
  M[1] = S2[0][1] - S1[0] * S1[1] / n_points;
  M[5] = S2[1][2] - S1[1] * S1[2] / n_points;
  M[2] = S2[0][2] - S1[0] * S1[2] / n_points;
  M[3] = M[1];
  M[6] = M[2];
  M[7] = M[5];
}

// eigen_old, geometry-inl.h:236-337: cyclic Jacobi with the Numerical-Recipes
// threshold schedule.  vout receives the rotation's rows as its columns
// (row-major here: vout[3 * r + c] = v[c][r]); dout the eigenvalues.  Both
// stay untouched when 50 sweeps do not clear the off-diagonal.
inline void refEigenOld(const double m[9], double dout[3], double vout[9]) {
  double R[9];
  for (int k = 0; k < 9; ++k) R[k] = m[k];
  auto Rr = [&](int r, int c) -> double& { return R[3 * r + c]; };
  const int n = 3;
  double b[3], z[3], d[3];
  double v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int ip = 0; ip < n; ++ip) {
    b[ip] = d[ip] = Rr(ip, ip);
    z[ip] = 0;
  }
  for (int i = 0; i < 50; ++i) {
    double sm = 0;
    for (int ip = 0; ip < n; ++ip)
      for (int iq = ip + 1; iq < n; ++iq) sm += std::abs(Rr(ip, iq));
    if (sm == 0.0) {
      for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) vout[3 * r + c] = v[c][r];
      for (int k = 0; k < 3; ++k) dout[k] = d[k];
      return;
    }
    const double tresh = (i < 3) ? 0.2 * sm / (n * n) : 0.0;
    for (int ip = 0; ip < n; ++ip) {
      for (int iq = ip + 1; iq < n; ++iq) {
        double g = 100.0 * std::abs(Rr(ip, iq));
        if (i > 3 && std::abs(d[ip]) + g == std::abs(d[ip]) && std::abs(d[iq]) + g == std::abs(d[iq])) {
          Rr(ip, iq) = 0.0;
        } else if (std::abs(Rr(ip, iq)) > tresh) {
          double h = d[iq] - d[ip];
          double t;
          if (std::abs(h) + g == std::abs(h)) {
            t = (Rr(ip, iq)) / h;
          } else {
            const double theta = 0.5 * h / (Rr(ip, iq));
            t = 1.0 / (std::abs(theta) + std::sqrt(1.0 + theta * theta));
            if (theta < 0.0) t = -t;
          }
          const double c = 1.0 / std::sqrt(1 + t * t);
          const double s = t * c;
          const double tau = s / (1.0 + c);
          h = t * Rr(ip, iq);
          z[ip] -= h;
          z[iq] += h;
          d[ip] -= h;
          d[iq] += h;
          Rr(ip, iq) = 0.0;
          auto rot = [&](double& x, double& y) {
            const double gg = x, hh = y;
            x = gg - s * (hh + gg * tau);
            y = hh + s * (gg - hh * tau);
          };
          for (int j = 0; j < ip; ++j) rot(Rr(j, ip), Rr(j, iq));
          for (int j = ip + 1; j < iq; ++j) rot(Rr(ip, j), Rr(j, iq));
          for (int j = iq + 1; j < n; ++j) rot(Rr(ip, j), Rr(iq, j));
          for (int j = 0; j < n; ++j) rot(v[j][ip], v[j][iq]);
        }
      }
    }
    for (int ip = 0; ip < n; ++ip) {
      b[ip] += z[ip];
      d[ip] = b[ip];
      z[ip] = 0.0;
    }
  }
}

// axisFromEigen (Matrix3 form), geometry-inl.h:339-366: columns 0 and 1 are
// the eigenvector rows of the largest and middle eigenvalue, column 2 their
// cross product.
inline void refAxisFromEigen(const double E[9], const double s[3], double axis[9]) {
  int mn, md, mx;
  if (s[0] > s[1]) {
    mx = 0;
    mn = 1;
  } else {
    mn = 0;
    mx = 1;
  }
  if (s[2] < s[mn]) {
    md = mn;
    mn = 2;
  } else if (s[2] > s[mx]) {
    md = mx;
    mx = 2;
  } else {
    md = 2;
  }
  double c0[3], c1[3];
  for (int k = 0; k < 3; ++k) {
    c0[k] = E[3 * mx + k];
    c1[k] = E[3 * md + k];
  }
  for (int k = 0; k < 3; ++k) {
    axis[3 * k] = c0[k];
    axis[3 * k + 1] = c1[k];
  }
  axis[2] = c0[1] * c1[2] - c0[2] * c1[1];
  axis[5] = c0[2] * c1[0] - c0[0] * c1[2];
  axis[8] = c0[0] * c1[1] - c0[1] * c1[0];
}

// FitImpl<S, OBBRSS<S>>::run, OBB half (BV_fitter-inl.h:323-345) with
// getExtentAndCenter_mesh (geometry-inl.h:147-182).
inline void refFitObb(const double* V, const int32_t* T, const uint32_t* idx, int n, RefNode& nd) {
  double M[9], s[3] = {0, 0, 0}, E[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  refCovariance(V, T, idx, n, M);
  refEigenOld(M, s, E);
  refAxisFromEigen(E, s, nd.axis);
  const double big = std::numeric_limits<double>::max();
  double mn[3] = {big, big, big}, mx[3] = {-big, -big, -big};
  for (int i = 0; i < n; ++i) {
    const int32_t* t = T + 3 * (size_t)idx[i];
    for (int j = 0; j < 3; ++j) {
      const double* p = V + 3 * (size_t)t[j];
      double proj[3];
      for (int k = 0; k < 3; ++k)
        proj[k] = (nd.axis[k] * p[0] + nd.axis[3 + k] * p[1]) + nd.axis[6 + k] * p[2];
      for (int k = 0; k < 3; ++k) {
        if (proj[k] > mx[k]) mx[k] = proj[k];
        if (proj[k] < mn[k]) mn[k] = proj[k];
      }
    }
  }
  double o[3];
  for (int k = 0; k < 3; ++k) o[k] = (mx[k] + mn[k]) / 2;
  for (int r = 0; r < 3; ++r) nd.To[r] = (nd.axis[3 * r] * o[0] + nd.axis[3 * r + 1] * o[1]) + nd.axis[3 * r + 2] * o[2];
  for (int k = 0; k < 3; ++k) nd.extent[k] = (mx[k] - mn[k]) / 2;
  nd.size = (nd.extent[0] * nd.extent[0] + nd.extent[1] * nd.extent[1]) + nd.extent[2] * nd.extent[2];
}

inline void buildRefTree(const double* V, const int32_t* T, int nt, std::vector<RefNode>& nodes,
                         std::vector<uint32_t>& prim) {
  nodes.clear();
  prim.resize(nt);
  for (int i = 0; i < nt; ++i) prim[i] = (uint32_t)i;
  if (nt <= 0) return;
  nodes.reserve(2 * (size_t)nt - 1);
  struct Task {
    int node, first, count;
  };
  std::vector<Task> tasks;
  nodes.emplace_back();
  tasks.push_back({0, 0, nt});
  while (!tasks.empty()) {
    const Task task = tasks.back();
    tasks.pop_back();
    uint32_t* cur = prim.data() + task.first;
    RefNode fitted;
    refFitObb(V, T, cur, task.count, fitted);
    fitted.first_primitive = task.first;
    fitted.num_primitives = task.count;
    fitted.first_child = 0;
    nodes[task.node] = fitted;
    if (task.count == 1) {
      nodes[task.node].first_child = -((int)cur[0] + 1);
      continue;
    }
    // computeSplitValue_mean on the first OBB axis
    const double sv[3] = {fitted.axis[0], fitted.axis[3], fitted.axis[6]};
    double c[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < task.count; ++i) {
      const int32_t* t = T + 3 * (size_t)cur[i];
      const double* p1 = V + 3 * (size_t)t[0];
      const double* p2 = V + 3 * (size_t)t[1];
      const double* p3 = V + 3 * (size_t)t[2];
      for (int k = 0; k < 3; ++k) c[k] += ((p1[k] + p2[k]) + p3[k]) / 3;
    }
    const double split_value = ((c[0] * sv[0] + c[1] * sv[1]) + c[2] * sv[2]) / task.count;
    int c1 = 0;
    for (int i = 0; i < task.count; ++i) {
      const int32_t* t = T + 3 * (size_t)cur[i];
      const double* p1 = V + 3 * (size_t)t[0];
      const double* p2 = V + 3 * (size_t)t[1];
      const double* p3 = V + 3 * (size_t)t[2];
      double p[3];
      for (int k = 0; k < 3; ++k) p[k] = ((p1[k] + p2[k]) + p3[k]) / 3.0;
      if (!(((sv[0] * p[0] + sv[1] * p[1]) + sv[2] * p[2]) > split_value)) {
        std::swap(cur[i], cur[c1]);
        ++c1;
      }
    }
    if (c1 == 0 || c1 == task.count) c1 = task.count / 2;
    const int left = (int)nodes.size();
    nodes.emplace_back();
    nodes.emplace_back();
    nodes[task.node].first_child = left;
    tasks.push_back({left + 1, task.first + c1, task.count - c1});
    tasks.push_back({left, task.first, c1});
  }
}

// overlap(R0, T0, OBB b1, OBB b2) on the FP64 nodes (OBB-inl.h:305-316).
inline bool refObbOverlap(const Mat3& R0, const double T0[3], const RefNode& b1, const RefNode& b2) {
  const double* A1 = b1.axis;
  const double* A2 = b2.axis;
  double R0b2[9];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c)
      R0b2[3 * r + c] = (R0.m[3 * r] * A2[c] + R0.m[3 * r + 1] * A2[3 + c]) + R0.m[3 * r + 2] * A2[6 + c];
  Mat3 R;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c)
      R.m[3 * r + c] = (A1[r] * R0b2[c] + A1[3 + r] * R0b2[3 + c]) + A1[6 + r] * R0b2[6 + c];
  double Tt[3];
  for (int r = 0; r < 3; ++r)
    Tt[r] = (((R0.m[3 * r] * b2.To[0] + R0.m[3 * r + 1] * b2.To[1]) + R0.m[3 * r + 2] * b2.To[2]) + T0[r]) - b1.To[r];
  double Tv[3];
  for (int c = 0; c < 3; ++c) Tv[c] = (Tt[0] * A1[c] + Tt[1] * A1[3 + c]) + Tt[2] * A1[6 + c];
  return !obbDisjoint(R, Tv, b1.extent, b2.extent);
}

// MeshIntersect (bvh_solver-inl.h:74-164) over the reference's own FP64 trees
// and FP64 vertices: contacts (b1, b2) in the order the reference adds them,
// at most max_contacts.
inline void meshIntersectRef(const RefNode* na, const double* Va, const int32_t* Ta, const RefNode* nb,
                             const double* Vb, const int32_t* Tb, const Mat3& R, const double T[3],
                             size_t max_contacts, std::vector<std::pair<int, int>>& contacts) {
  contacts.clear();
  if (max_contacts == 0) return;
  auto vtx = [](const double* V, const int32_t* Tr, int t, int k) {
    const double* p = V + 3 * (size_t)Tr[3 * (size_t)t + k];
    return P3{p[0], p[1], p[2]};
  };
  std::vector<std::pair<int, int>> stack;
  stack.emplace_back(0, 0);
  while (!stack.empty()) {
    const std::pair<int, int> task = stack.back();
    stack.pop_back();
    const RefNode& a = na[task.first];
    const RefNode& b = nb[task.second];
    if (!refObbOverlap(R, T, a, b)) continue;
    const bool la = a.first_child < 0, lb = b.first_child < 0;
    if (la && lb) {
      const int ta = -(a.first_child + 1), tb = -(b.first_child + 1);
      if (intersectTriangle(vtx(Va, Ta, ta, 0), vtx(Va, Ta, ta, 1), vtx(Va, Ta, ta, 2), vtx(Vb, Tb, tb, 0),
                            vtx(Vb, Tb, tb, 1), vtx(Vb, Tb, tb, 2), R, T)) {
        contacts.emplace_back(ta, tb);
        if (contacts.size() >= max_contacts) return;
      }
      continue;
    }
    const bool go_a = lb || (!la && a.size > b.size);
    if (go_a) {
      stack.emplace_back(a.first_child, task.second);
      stack.emplace_back(a.first_child + 1, task.second);
    } else {
      stack.emplace_back(task.first, b.first_child);
      stack.emplace_back(task.first, b.first_child + 1);
    }
  }
}

// Every colliding triangle pair by brute force (test support for small meshes).
inline void allPairs(const float* tri_a, int na, const float* tri_b, int nb, const Mat3& R, const double T[3],
                     std::vector<std::pair<int, int>>& contacts) {
  contacts.clear();
  auto vtx = [](const float* tris, int t, int k) {
    const float* p = tris + 12 * (size_t)t + 4 * k;
    return P3{p[0], p[1], p[2]};
  };
  for (int i = 0; i < na; ++i)
    for (int j = 0; j < nb; ++j)
      if (intersectTriangle(vtx(tri_a, i, 0), vtx(tri_a, i, 1), vtx(tri_a, i, 2), vtx(tri_b, j, 0), vtx(tri_b, j, 1),
                            vtx(tri_b, j, 2), R, T))
        contacts.emplace_back(i, j);
}

}  // namespace orc
