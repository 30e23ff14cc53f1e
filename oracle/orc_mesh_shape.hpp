// ORACLE — test infrastructure only.
//
// FP64 restatement of fcl::collide on a triangle mesh (BVHModel<OBBRSS>)
// against a shape with penetration off: OrientedNodeBVHSolver::
// MeshShapeIntersect (narrowphase/detail/traversal/collision/bvh_solver-inl.h:
// 6-72) and the shape-triangle tests it reaches through
// ShapePairIntersectSolver::ShapeSimplexIntersect
// (shape_pair_intersect-inl.h:137-160) and GJKSolver::shapeTriangleIntersect
// with the triangle's transform (gjk_solver-inl.h:451-591):
//   sphere      sphereTriangleIntersect, sphere_triangle-inl.h:52-191
//   box         boxTriangleIntersect, box_triangle-inl.h:1-147
//   others      MPR::Intersect on (shape, triangle) (use_mpr_if_no_contact)
// The mesh is the frame; the shape is posed by (R, t) in it.  The tree is an
// input (the library's flattened OBB tree).  The shape's bounding box only
// prunes: here a box along the shape's own axes that bounds it (the reference
// fits hulls by principal axes), which leaves the colliding set and the
// depth-first order of its leaves unchanged.
#pragma once

#include <algorithm>
#include <cmath>
#include <limits>
#include <vector>

#include "orc_convex.hpp"
#include "orc_mesh.hpp"

namespace orc {

// sphere_triangle-inl.h:52-78
inline double segmentSqrDistance(const V3& from, const V3& to, const V3& p, V3& nearest) {
  V3 diff = p - from;
  const V3 v = to - from;
  double t = dot(v, diff);
  if (t > 0) {
    const double vv = dot(v, v);
    if (t < vv) {
      t /= vv;
      diff = diff - v * t;
    } else {
      t = 1;
      diff = diff - v;
    }
  } else {
    t = 0;
  }
  nearest = from + v * t;
  return dot(diff, diff);
}

// sphere_triangle-inl.h:81-104
inline bool projectInTriangle(const V3& p1, const V3& p2, const V3& p3, const V3& normal, const V3& p) {
  const V3 e1 = p2 - p1, e2 = p3 - p2, e3 = p1 - p3;
  const double r1 = dot(cross(e1, normal), p - p1);
  const double r2 = dot(cross(e2, normal), p - p2);
  const double r3 = dot(cross(e3, normal), p - p3);
  return (r1 > 0 && r2 > 0 && r3 > 0) || (r1 <= 0 && r2 <= 0 && r3 <= 0);
}

// sphereTriangleIntersect, sphere_triangle-inl.h:107-191 (the boolean)
inline bool sphereTriangleIntersect(double radius, const V3& center, const V3& P1, const V3& P2, const V3& P3) {
  V3 normal = normalized(cross(P2 - P1, P3 - P1));
  const double rt = radius + std::numeric_limits<double>::epsilon();
  double dist = dot(center - P1, normal);
  if (dist < 0) {
    dist = -dist;
    normal = -normal;
  }
  if (!(dist < rt)) return false;
  bool has = false;
  V3 cp;
  if (projectInTriangle(P1, P2, P3, normal, center)) {
    has = true;
    cp = center - normal * dist;
  } else {
    const double r2 = rt * rt;
    V3 near;
    if (segmentSqrDistance(P1, P2, center, near) < r2) { has = true; cp = near; }
    if (segmentSqrDistance(P2, P3, center, near) < r2) { has = true; cp = near; }
    if (segmentSqrDistance(P3, P1, center, near) < r2) { has = true; cp = near; }
  }
  if (!has) return false;
  return sqn(cp - center) < rt * rt;
}

// box_triangle-inl.h:9-69: the three axes box_axis x edge for one triangle edge
inline bool boxTriangleSeparatedByEdge(const V3& h, const V3& e, const V3& v0, const V3& v1) {
  const double ex = e[0], ey = e[1], ez = e[2];
  const double ax = std::abs(ex), ay = std::abs(ey), az = std::abs(ez);
  auto test = [](double r, double p0, double p1) {
    if (p0 < p1) return p0 > r || p1 < -r;
    return p1 > r || p0 < -r;
  };
  if (test(h[1] * az + h[2] * ay, v0[1] * ez - v0[2] * ey, v1[1] * ez - v1[2] * ey)) return true;
  if (test(h[0] * az + h[2] * ax, v0[0] * ez - v0[2] * ex, v1[0] * ez - v1[2] * ex)) return true;
  if (test(h[0] * ay + h[1] * ax, v0[0] * ey - v0[1] * ex, v1[0] * ey - v1[1] * ex)) return true;
  return false;
}

// detectBoxTriangleOverlap, box_triangle-inl.h:71-119 (triangle in the box's frame)
inline bool detectBoxTriangleOverlap(const V3& h, const V3& v0, const V3& v1, const V3& v2) {
  for (int i = 0; i < 3; ++i) {
    const double mn = std::min(v0[i], std::min(v1[i], v2[i])), mx = std::max(v0[i], std::max(v1[i], v2[i]));
    if (mx < -h[i] || mn > h[i]) return false;
  }
  const V3 e0 = v1 - v0, e1 = v2 - v1, e2 = v0 - v2;
  if (boxTriangleSeparatedByEdge(h, e0, v0, v2)) return false;
  if (boxTriangleSeparatedByEdge(h, e1, v1, v0)) return false;
  if (boxTriangleSeparatedByEdge(h, e2, v0, v1)) return false;
  const V3 n = cross(e0, e1);
  V3 pmin, pmax;
  for (int i = 0; i < 3; ++i) {
    if (n[i] > 0) {
      pmin[i] = -h[i] - v0[i];
      pmax[i] = h[i] - v0[i];
    } else {
      pmin[i] = h[i] - v0[i];
      pmax[i] = -h[i] - v0[i];
    }
  }
  return dot(n, pmin) <= 0 && dot(n, pmax) >= 0;
}

// The shape-triangle boolean fcl::collide uses for one leaf.  X: the shape's
// pose in the mesh frame; P: the triangle in the mesh frame.
inline bool shapeTriangleIntersect(const Shape& s, const Iso& X, const float* tri_xyzw, const SolverParams& sp) {
  const V3 P1(tri_xyzw[0], tri_xyzw[1], tri_xyzw[2]), P2(tri_xyzw[4], tri_xyzw[5], tri_xyzw[6]),
      P3(tri_xyzw[8], tri_xyzw[9], tri_xyzw[10]);
  // the triangle in the shape's frame: tf1^-1 * tf2 (tf2 = identity)
  Iso inv;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) inv.R[3 * r + c] = X.R[3 * c + r];
  inv.t = -inv.rot(X.t);
  if (s.type == kSphere) return sphereTriangleIntersect(s.p[0], X.t, P1, P2, P3);
  if (s.type == kBox) {
    const V3 h = V3(s.p[0], s.p[1], s.p[2]) * 0.5;
    return detectBoxTriangleOverlap(h, inv.apply(P1), inv.apply(P2), inv.apply(P3));
  }
  Shape tri;
  tri.type = kTriangle;
  tri.verts = tri_xyzw;
  tri.nv = 3;
  tri.interior = (P1 + P2 + P3) / 3.0;
  MinkDiff md;
  md.s0 = &s;
  md.s1 = &tri;
  md.to0 = inv;
  MPR mpr(sp.gjk_max_iter, sp.gjk_tol);
  return mpr.Intersect(md) == MPRStatus::Intersect;
}

// A box along the shape's own axes that bounds it, in the mesh frame.
inline MeshNode shapeBox(const Shape& s, const Iso& X) {
  MeshNode n{};
  double c[3] = {0, 0, 0}, e[3] = {0, 0, 0};
  bool own_axes = true;
  switch (s.type) {
    case kBox: for (int i = 0; i < 3; ++i) e[i] = 0.5 * s.p[i]; break;
    case kSphere: for (int i = 0; i < 3; ++i) e[i] = s.p[0]; own_axes = false; break;
    case kCapsule: e[0] = e[1] = s.p[0]; e[2] = 0.5 * s.p[1] + s.p[0]; break;
    case kCylinder: e[0] = e[1] = s.p[0]; e[2] = 0.5 * s.p[1]; break;
    default: {
      double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
      for (int k = 0; k < s.nv; ++k)
        for (int i = 0; i < 3; ++i) {
          lo[i] = std::min(lo[i], (double)s.verts[4 * k + i]);
          hi[i] = std::max(hi[i], (double)s.verts[4 * k + i]);
        }
      for (int i = 0; i < 3; ++i) { c[i] = 0.5 * (lo[i] + hi[i]); e[i] = 0.5 * (hi[i] - lo[i]); }
    }
  }
  const V3 cw = X.apply(V3(c[0], c[1], c[2]));
  for (int r = 0; r < 3; ++r)
    for (int k = 0; k < 3; ++k) n.axis[3 * r + k] = own_axes ? (float)X.R[3 * r + k] : (r == k ? 1.f : 0.f);
  for (int i = 0; i < 3; ++i) {
    n.center[i] = (float)cw[i];
    // FP32 storage: widen by the rounding of centre, axes and extent
    n.extent[i] = (float)(e[i] * (1 + 1e-6) + 1e-6 * (1.0 + std::abs(cw[i])));
  }
  n.child = 0;
  return n;
}

// MeshShapeIntersect, bvh_solver-inl.h:6-72: depth first from the root, the
// second child popped first; leaf contacts until max_contacts.
inline void meshShapeIntersect(const MeshNode* nodes, const float* tris, const Shape& s, const Iso& X,
                               size_t max_contacts, const SolverParams& sp, std::vector<int>& contacts) {
  contacts.clear();
  if (max_contacts == 0) return;
  const MeshNode sb = shapeBox(s, X);
  Mat3 I;
  for (int k = 0; k < 9; ++k) I.m[k] = (k % 4 == 0) ? 1.0 : 0.0;
  const double T0[3] = {0, 0, 0};
  std::vector<int> stack{0};
  while (!stack.empty()) {
    const int id = stack.back();
    stack.pop_back();
    const MeshNode& n = nodes[id];
    if (!obbOverlap(I, T0, sb, n)) continue;
    if (n.child >= 0) {
      stack.push_back(n.child);
      stack.push_back(n.child + 1);
      continue;
    }
    const int t = -(n.child + 1);
    if (shapeTriangleIntersect(s, X, tris + 12 * (size_t)t, sp)) {
      contacts.push_back(t);
      if (contacts.size() >= max_contacts) return;
    }
  }
}

// ---------------------------------------------------- penetration contacts --
// ShapePairIntersectSolver::ShapeSimplexIntersect with penetration on
// (narrowphase/detail/shape_pair_intersect-inl.h:132-170) for a triangle: the
// contact of shapeTriangleIntersect (gjk_solver-inl.h:305-375, 405-449), its
// normal reversed by the mesh-shape contact meta (bvh_solver-inl.h:56-61,
// shape_pair_intersect-inl.h:19-26).  pos and normal in the mesh frame.
struct MsContact {
  int tri = -1;
  V3 pos, normal;
  double depth = 0;
  int epa_status = -1;  // -1: closed form (sphere)
};

// sphereTriangleIntersect with its outputs (sphere_triangle-inl.h:107-191).
inline bool sphereTriangleContact(double radius, const V3& center, const V3& P1, const V3& P2, const V3& P3, V3& pos,
                                  V3& normal_out, double& depth) {
  V3 normal = normalized(cross(P2 - P1, P3 - P1));
  const double rt = radius + std::numeric_limits<double>::epsilon();
  double dist = dot(center - P1, normal);
  if (dist < 0) {
    dist = -dist;
    normal = -normal;
  }
  if (!(dist < rt)) return false;
  bool has = false;
  V3 cp;
  if (projectInTriangle(P1, P2, P3, normal, center)) {
    has = true;
    cp = center - normal * dist;
  } else {
    const double r2 = rt * rt;
    V3 near;
    if (segmentSqrDistance(P1, P2, center, near) < r2) { has = true; cp = near; }
    if (segmentSqrDistance(P2, P3, center, near) < r2) { has = true; cp = near; }
    if (segmentSqrDistance(P3, P1, center, near) < r2) { has = true; cp = near; }
  }
  if (!has) return false;
  const V3 ctc = cp - center;
  const double d2 = sqn(ctc);
  if (!(d2 < rt * rt)) return false;
  pos = cp;
  if (d2 > 0) {
    normal_out = normalized(ctc);
    depth = -(radius - std::sqrt(d2));
  } else {
    normal_out = -normal;
    depth = -radius;
  }
  return true;
}

inline bool shapeTriangleContact(const Shape& s, const Iso& X, const float* tri_xyzw, const SolverParams& sp,
                                 MsContact& c) {
  const V3 P1(tri_xyzw[0], tri_xyzw[1], tri_xyzw[2]), P2(tri_xyzw[4], tri_xyzw[5], tri_xyzw[6]),
      P3(tri_xyzw[8], tri_xyzw[9], tri_xyzw[10]);
  if (s.type == kSphere) {
    V3 pos, nrm;
    double depth;
    if (!sphereTriangleContact(s.p[0], X.t, P1, P2, P3, pos, nrm, depth)) return false;
    c.pos = pos;
    c.normal = -nrm;
    c.depth = depth;
    c.epa_status = -1;
    return true;
  }
  Iso inv;
  for (int r = 0; r < 3; ++r)
    for (int k = 0; k < 3; ++k) inv.R[3 * r + k] = X.R[3 * k + r];
  inv.t = -inv.rot(X.t);
  Shape tri;
  tri.type = kTriangle;
  tri.verts = tri_xyzw;
  tri.nv = 3;
  tri.interior = (P1 + P2 + P3) / 3.0;
  MinkDiff md;
  md.s0 = &s;
  md.s1 = &tri;
  md.to0 = inv;
  GJK gjk(sp.gjk_max_iter, sp.gjk_tol);
  Simplex smp;
  if (gjk.Evaluate(md, smp, V3(-1, 0, 0), nullptr) != GJKStatus::Intersect) return false;
  EPA epa(sp.epa_max_faces, sp.epa_max_iter, sp.epa_tol);
  double depth = 0;
  V3 p0, p1;
  const EPAStatus es = epa.Evaluate(smp, md, depth, p0, p1);
  if (es == EPAStatus::Failed) return false;
  V3 n = p0 - p1;
  if (sqn(n) <= 0) n = V3(0, 0, 1);
  else normalize(n);
  c.pos = X.apply((p0 + p1) * 0.5);
  c.normal = -X.rot(n);
  c.depth = depth;
  c.epa_status = (int)es;
  return true;
}

// MeshShapeIntersect with penetration on: the traversal of meshShapeIntersect,
// each leaf adding its contact.
inline void meshShapeContacts(const MeshNode* nodes, const float* tris, const Shape& s, const Iso& X,
                              size_t max_contacts, const SolverParams& sp, std::vector<MsContact>& contacts) {
  contacts.clear();
  if (max_contacts == 0) return;
  const MeshNode sb = shapeBox(s, X);
  Mat3 I;
  for (int k = 0; k < 9; ++k) I.m[k] = (k % 4 == 0) ? 1.0 : 0.0;
  const double T0[3] = {0, 0, 0};
  std::vector<int> stack{0};
  while (!stack.empty()) {
    const int id = stack.back();
    stack.pop_back();
    const MeshNode& n = nodes[id];
    if (!obbOverlap(I, T0, sb, n)) continue;
    if (n.child >= 0) {
      stack.push_back(n.child);
      stack.push_back(n.child + 1);
      continue;
    }
    const int t = -(n.child + 1);
    MsContact c;
    if (shapeTriangleContact(s, X, tris + 12 * (size_t)t, sp, c)) {
      c.tri = t;
      contacts.push_back(c);
      if (contacts.size() >= max_contacts) return;
    }
  }
}

}  // namespace orc
