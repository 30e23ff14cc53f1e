// ORACLE — test infrastructure only.
//
// FP64 restatement of mind-fcl's OBB BVH-vs-BVH boolean collision
// (OrientedNodeBVHSolver::MeshIntersect with penetration off): the OBB overlap
// test, the triangle-triangle separating-axis test, and the traversal order.
// The BVH itself is an input (the flattened tree the GPU library builds), so
// the oracle and the GPU traverse the same tree; the set of colliding triangle
// pairs does not depend on the tree.
#pragma once

#include <cmath>
#include <cstdint>
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
