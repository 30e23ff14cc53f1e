// ORACLE — test infrastructure only.
//
// FP64 restatement of the closed-form shape-pair solvers fcl::collide uses
// instead of MPR / GJK+EPA for sphere pairs (ShapeIntersectIndepImpl
// specialisations, include/fcl/narrowphase/detail/gjk_solver-inl.h:209-218):
//   sphereSphereIntersect    primitive_shape_algorithm/sphere_sphere-inl.h:48-66
//   sphereCapsuleIntersect   primitive_shape_algorithm/sphere_capsule-inl.h:49-63, 70-100
//   sphereBoxIntersect       primitive_shape_algorithm/sphere_box-inl.h:59-172
//   sphereCylinderIntersect  primitive_shape_algorithm/sphere_cylinder-inl.h:60-201
// The reversed pairs call the same solver with the shapes swapped and flip the
// contact normal (gjk_solver-inl.h:190-201).  Frames: shape a at the origin,
// shape b posed by `pose` in a's frame, as the batch API states pairs.
// Contact: normal = escape direction of shape b, pos, depth (contact_point.h).
// Box-box (boxBoxIntersect) is not restated: the library answers box pairs by
// MPR / GJK+EPA.
#pragma once
#include "orc_convex.hpp"

namespace orc {

struct AContact {
  bool hit = false;
  V3 normal, pos;
  double depth = 0;
  double separation = -1;  // centre-based separation when not hit
};

// 16 eps of the scalar type (constants<S>::eps(), the reference's noise floor).
constexpr double kAnalyticEps = 16 * 2.220446049250313e-16;

// sphere_sphere-inl.h:48-66; c1 at the origin, c2 = t
inline AContact sphereSphere(double r1, double r2, const V3& c2) {
  AContact c;
  const V3 diff = c2;
  const double len = norm(diff);
  if (len > r1 + r2) { c.separation = len - (r1 + r2); return c; }
  c.hit = true;
  c.normal = len > 0 ? diff / len : diff;
  c.pos = diff * (r1 / (r1 + r2));
  c.depth = r1 + r2 - len;
  return c;
}

// sphere_capsule-inl.h:49-63
inline V3 segmentPointClosestToPoint(const V3& p, const V3& s1, const V3& s2) {
  const V3 v = s2 - s1, w = p - s1;
  const double c1 = dot(w, v), c2 = dot(v, v);
  if (c1 <= 0) return s1;
  if (c2 <= c1) return s2;
  return s1 + v * (c1 / c2);
}

// sphere_capsule-inl.h:70-100; sphere at the origin (frame F = a's frame),
// capsule posed by X_FC
inline AContact sphereCapsule(double rs, double rc, double lz, const Iso& X_FC, const V3& sphere_centre_F) {
  AContact c;
  const V3 pos1(0, 0, 0.5 * lz), pos2(0, 0, -0.5 * lz);
  const V3 s_c = X_FC.rotT(sphere_centre_F - X_FC.t);   // X_FC^-1 * centre
  const V3 sp = segmentPointClosestToPoint(s_c, pos1, pos2);
  const V3 diff = s_c - sp;
  const double distance = norm(diff) - rs - rc;
  if (distance > 0) { c.separation = distance; return c; }
  const V3 local_normal = -normalized(diff);
  c.hit = true;
  c.normal = X_FC.rot(local_normal);
  c.pos = X_FC.apply(sp + local_normal * distance);
  c.depth = -distance;
  return c;
}

// sphere_box-inl.h:59-172; sphere posed by X_FS, box posed by X_FB
inline AContact sphereBox(double r, const V3& side, const Iso& X_FB, const V3& sphere_centre_F) {
  AContact c;
  const V3 p_BC = X_FB.rotT(sphere_centre_F - X_FB.t);
  const V3 half = side / 2;
  V3 p_BN = p_BC;
  bool clamped = false;
  for (int i = 0; i < 3; ++i) {
    if (p_BC[i] < -half[i]) { clamped = true; p_BN[i] = -half[i]; }
    if (p_BC[i] > half[i]) { clamped = true; p_BN[i] = half[i]; }
  }
  const V3 p_CN_B = p_BN - p_BC;
  const double sq = sqn(p_CN_B);
  if (sq > r * r) { c.separation = std::sqrt(sq) - r; return c; }
  c.hit = true;
  V3 n_SB_B, p_BP;
  if (clamped && sq > kAnalyticEps * kAnalyticEps) {
    const double distance = std::sqrt(sq);
    n_SB_B = p_CN_B / distance;
    c.depth = r - distance;
    p_BP = p_BN + n_SB_B * (c.depth * 0.5);
  } else {
    double min_distance = std::numeric_limits<double>::infinity();
    int min_axis = -1;
    for (int i = 0; i < 3; ++i) {
      const double dist = p_BC[i] >= 0 ? half[i] - p_BC[i] : p_BC[i] + half[i];
      if (dist + kAnalyticEps < min_distance) { min_distance = dist; min_axis = i; }
    }
    n_SB_B = V3(0, 0, 0);
    n_SB_B[min_axis] = p_BC[min_axis] >= 0 ? -1 : 1;
    c.depth = min_distance + r;
    p_BP = p_BC + n_SB_B * ((r - min_distance) / 2);
  }
  c.normal = X_FB.rot(n_SB_B);
  c.pos = X_FB.apply(p_BP);
  return c;
}

// sphere_cylinder-inl.h:60-201; sphere posed by X_FS, cylinder by X_FC
inline AContact sphereCylinder(double rs, double rc, double lz, const Iso& X_FC, const V3& sphere_centre_F) {
  AContact c;
  const V3 p_CS = X_FC.rotT(sphere_centre_F - X_FC.t);
  V3 p_CN = p_CS;
  bool outside = false;
  const double half_h = lz / 2;
  if (p_CS[2] > half_h) { outside = true; p_CN[2] = half_h; }
  else if (p_CS[2] < -half_h) { outside = true; p_CN[2] = -half_h; }
  double rx = p_CS[0], ry = p_CS[1];
  const double sqxy = rx * rx + ry * ry;
  if (sqxy > rc * rc) {
    outside = true;
    const double k = rc / std::sqrt(sqxy);
    rx *= k;
    ry *= k;
    p_CN[0] = rx;
    p_CN[1] = ry;
  }
  const V3 p_SN_C = p_CN - p_CS;
  const double sq = sqn(p_SN_C);
  if (sq > rs * rs) { c.separation = std::sqrt(sq) - rs; return c; }
  c.hit = true;
  V3 n, p_CP;
  if (outside && sq > kAnalyticEps * kAnalyticEps) {
    const double d_NS = std::sqrt(sq);
    n = p_SN_C / d_NS;
    c.depth = rs - d_NS;
    p_CP = p_CN + n * (c.depth * 0.5);
  } else {
    const double face_distance = p_CS[2] >= 0 ? lz / 2 - p_CS[2] : p_CS[2] + lz / 2;
    const double d_xy = std::sqrt(p_CS[0] * p_CS[0] + p_CS[1] * p_CS[1]);
    const double barrel_distance = rc - d_xy;
    if (barrel_distance < face_distance - kAnalyticEps) {
      if (d_xy > kAnalyticEps) {
        n = V3(-p_CS[0] / d_xy, -p_CS[1] / d_xy, 0);
        c.depth = rs + barrel_distance;
      } else {
        n = V3(-1, 0, 0);
        c.depth = rs + rc;
      }
      p_CP = p_CS + n * ((rs - barrel_distance) / 2);
    } else {
      n = V3(0, 0, p_CS[2] >= 0 ? -1 : 1);
      c.depth = face_distance + rs;
      p_CP = p_CS + n * ((rs - face_distance) / 2);
    }
  }
  c.normal = X_FC.rot(n);
  c.pos = X_FC.apply(p_CP);
  return c;
}

// The solver fcl::collide picks for (a, b), with a at the origin and b posed
// by `pose`; false when the pair has no closed-form solver here.
inline bool analyticIntersect(const Shape& a, const Shape& b, const Iso& pose, AContact& out) {
  const bool sa = a.type == kSphere, sb = b.type == kSphere;
  if (!sa && !sb) return false;
  const Shape& other = sa ? b : a;
  if (sa && sb) {
    out = sphereSphere(a.p[0], b.p[0], pose.t);
    return true;
  }
  if (other.type != kCapsule && other.type != kBox && other.type != kCylinder) return false;
  if (sa) {
    // sphere a at the origin, other shape b posed by `pose`
    const V3 centre(0, 0, 0);
    if (other.type == kCapsule) out = sphereCapsule(a.p[0], other.p[0], other.p[1], pose, centre);
    else if (other.type == kBox) out = sphereBox(a.p[0], V3(other.p[0], other.p[1], other.p[2]), pose, centre);
    else out = sphereCylinder(a.p[0], other.p[0], other.p[1], pose, centre);
    return true;
  }
  // other shape a at the origin, sphere b at pose.t: the solver runs with the
  // sphere first, then the normal flips (gjk_solver-inl.h:190-201)
  Iso I;
  for (int k = 0; k < 9; ++k) I.R[k] = (k % 4 == 0) ? 1.0 : 0.0;
  I.t = V3(0, 0, 0);
  if (other.type == kCapsule) out = sphereCapsule(b.p[0], other.p[0], other.p[1], I, pose.t);
  else if (other.type == kBox) out = sphereBox(b.p[0], V3(other.p[0], other.p[1], other.p[2]), I, pose.t);
  else out = sphereCylinder(b.p[0], other.p[0], other.p[1], I, pose.t);
  out.normal = -out.normal;
  return true;
}

}  // namespace orc
