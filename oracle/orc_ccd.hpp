// ORACLE — test infrastructure only.
//
// FP64 restatement of the reference's translational continuous collision for
// shape pairs (fcl::translational_ccd, narrowphase/continuous_collision-inl.h:
// 20-37, through ShapePairTranslationalCollisionSolver::RunShapePair,
// narrowphase/detail/ccd/shape_pair_ccd-inl.h:57-160):
//
//   * the boolean and the one-sample time of collision by MPR on the
//     Minkowski difference of shape 1 swept along its displacement and shape 2
//     (TranslationalCollisionGJK, narrowphase/detail/ccd/gjk_ccd-inl.h:7-187);
//   * the time-of-collision interval of two boxes moving apart along one
//     axis, by the 15 box axes (BoxPairTranslationalCCD::IsDisjoint,
//     narrowphase/detail/ccd/box_pair_ccd-inl.h:10-393), used for box-box
//     pairs and as the box pre-check of the approximate request.
//
// The pair is posed in shape 1's frame (tf1 = identity, tf2 = the pair's
// pose), the displacement's axis is a unit vector in shape 1's frame.
#pragma once
#include <algorithm>
#include <cmath>
#include <limits>

#include "orc_convex.hpp"

namespace orc {

// TimeOfCollisionRequestType (narrowphase/detail/ccd/ccd_request.h:11-17).
enum class TocRequest : int { NotRequested = 0, BoxApproximate = 1, OneTocSample = 2 };

struct Interval {  // ccd_typedef.h:18-37
  double lo = -1.0, hi = -1.0;
  void intersect(const Interval& r) {
    lo = std::max(lo, r.lo);
    hi = std::min(hi, r.hi);
  }
  bool empty(double tol) const { return lo > hi + tol; }
};

// BoxPairTranslationalCCD::CheckEmptyTocIntervalOnAxis, scalar form
// (box_pair_ccd-inl.h:10-42): box 1 of half range h1 moving by |d| (sign
// `pos`) against box 2 of half range h2 centred at `off`; unscaled interval.
inline bool boxAxisEmpty(double h1, double abs_d, bool pos, double h2, double off, Interval& toc) {
  const double b1_lb = pos ? (-h1) : (-h1 - abs_d);
  const double b1_ub = pos ? (h1 + abs_d) : h1;
  const double b2_lb = off - h2;
  const double b2_ub = off + h2;
  if (b1_lb > b2_ub || b2_lb > b1_ub) return true;
  if (pos) {
    toc.lo = std::max(0.0, -h1 + b2_lb);
    toc.hi = std::min(abs_d, h1 + b2_ub);
  } else {
    toc.lo = std::max(0.0, -h1 - b2_ub);
    toc.hi = std::min(abs_d, h1 - b2_lb);
  }
  return false;
}

// The signed-displacement overload (box_pair_ccd-inl.h:87-97).
inline bool boxAxisEmptySigned(double h1, double d, double h2, double off, Interval& toc) {
  const bool pos = d > 0;
  return boxAxisEmpty(h1, pos ? d : -d, pos, h2, off, toc);
}

// Three axes at once, interval scaled to [0, 1] (box_pair_ccd-inl.h:44-85).
inline bool boxAxes3Empty(const double h1[3], const double d[3], const double h2[3], const double off[3],
                          Interval& toc, double zero_tol) {
  double b1_lb[3], b1_ub[3], b2_lb[3], b2_ub[3];
  bool pos[3];
  for (int k = 0; k < 3; ++k) {
    pos[k] = d[k] > 0.0;
    b1_lb[k] = pos[k] ? -h1[k] : (-h1[k] + d[k]);
    b1_ub[k] = pos[k] ? (h1[k] + d[k]) : h1[k];
    b2_lb[k] = off[k] - h2[k];
    b2_ub[k] = off[k] + h2[k];
  }
  for (int k = 0; k < 3; ++k)
    if (b1_lb[k] > b2_ub[k]) return true;
  for (int k = 0; k < 3; ++k)
    if (b2_lb[k] > b1_ub[k]) return true;
  double lo = -std::numeric_limits<double>::infinity(), hi = std::numeric_limits<double>::infinity();
  for (int k = 0; k < 3; ++k) {
    const double raw_lo = pos[k] ? (-h1[k] + b2_lb[k]) : (-h1[k] - b2_ub[k]);
    const double raw_hi = pos[k] ? (h1[k] + b2_ub[k]) : (h1[k] - b2_lb[k]);
    const double inv = 1.0 / std::max(std::abs(d[k]), zero_tol);
    lo = std::max(lo, std::max(raw_lo * inv, 0.0));
    hi = std::min(hi, std::min(raw_hi * inv, 1.0));
  }
  toc.lo = lo;
  toc.hi = hi;
  return toc.empty(0.0);
}

// ScaleIntervalBoxDisjoint (box_pair_ccd-inl.h:99-110).
inline void boxScale(Interval& t, double abs_d, double zero_tol) {
  if (abs_d < zero_tol) {
    t.lo = 0;
    t.hi = 1;
  } else {
    t.lo /= abs_d;
    t.hi /= abs_d;
  }
}

// isDisjointArray (box_pair_ccd-inl.h:112-214): box 1 (half sizes h1, axes
// of its frame) moving by unit_axis * dist, box 2 of half sizes h2 with
// rotation R (row-major, box 2 in box 1) and centre t; the time interval in
// [0, 1] when not disjoint.
inline bool boxPairDisjoint(const double h1[3], const V3& unit_axis, double dist, const double R[9], const V3& t,
                            const double h2[3], double zero_tol, Interval& iv) {
  double Ra[9];
  for (int k = 0; k < 9; ++k) Ra[k] = std::abs(R[k]);
  iv.lo = 0.0;
  iv.hi = 1.0;
  {  // box 1's axes
    double d[3], h2p[3], off[3];
    for (int k = 0; k < 3; ++k) {
      d[k] = unit_axis[k] * dist;
      h2p[k] = (Ra[3 * k] * h2[0] + Ra[3 * k + 1] * h2[1]) + Ra[3 * k + 2] * h2[2];
      off[k] = t[k];
    }
    Interval a;
    if (boxAxes3Empty(h1, d, h2p, off, a, zero_tol)) return true;
    iv.intersect(a);
    if (iv.empty(0.0)) return true;
  }
  {  // box 2's axes
    double h1p[3], d[3], off[3];
    for (int k = 0; k < 3; ++k) {
      h1p[k] = (Ra[k] * h1[0] + Ra[3 + k] * h1[1]) + Ra[6 + k] * h1[2];
      const double u = (R[k] * unit_axis[0] + R[3 + k] * unit_axis[1]) + R[6 + k] * unit_axis[2];
      d[k] = u * dist;
      off[k] = (R[k] * t[0] + R[3 + k] * t[1]) + R[6 + k] * t[2];
    }
    Interval a;
    if (boxAxes3Empty(h1p, d, h2, off, a, zero_tol)) return true;
    iv.intersect(a);
    if (iv.empty(0.0)) return true;
  }
  for (int k = 0; k < 3; ++k)
    for (int i = 0; i < 3; ++i) {
      // e_k x (column i of R), not unit, possibly zero
      const V3 c(R[i], R[3 + i], R[6 + i]);
      V3 e(0, 0, 0);
      e[k] = 1.0;
      const V3 a = cross(e, c);
      const V3 aa(std::abs(a.x), std::abs(a.y), std::abs(a.z));
      const double h1a = dot(aa, V3(h1[0], h1[1], h1[2]));
      const double off = dot(a, t);
      const V3 a2 = V3((R[0] * a.x + R[3] * a.y) + R[6] * a.z, (R[1] * a.x + R[4] * a.y) + R[7] * a.z,
                       (R[2] * a.x + R[5] * a.y) + R[8] * a.z);
      const V3 a2a(std::abs(a2.x), std::abs(a2.y), std::abs(a2.z));
      const double h2a = dot(a2a, V3(h2[0], h2[1], h2[2]));
      const double proj = dot(a, unit_axis);
      const bool pos = proj > 0;
      const double abs_d = pos ? proj * dist : -proj * dist;
      Interval s;
      if (boxAxisEmpty(h1a, abs_d, pos, h2a, off, s)) return true;
      boxScale(s, abs_d, zero_tol);
      iv.intersect(s);
      if (iv.empty(0.0)) return true;
    }
  return false;
}

// computeOneTocSampleForIntersection (gjk_ccd-inl.h:106-187): the time of
// collision at the origin's barycentric weights in the final MPR portal
// tetrahedron, each vertex at phase 1 if its direction points along the
// displacement, else 0 (the interior point at 0.5).
inline double tocSample(const V3& disp, const MPRPortal& P) {
  constexpr double v0_phase = 0.5;
  const V3& v0 = P.v0;
  if (P.count < 1) return v0_phase;
  const V3& v1 = P.v[0];
  if (P.count < 2) {
    const double n0 = norm(v0), n1 = norm(v1);
    const double n01 = n0 + n1;
    if (n01 <= 0.0) return v0_phase;
    const double inv = 1.0 / n01;
    const double w0 = n1 * inv, w1 = n0 * inv;
    const double ph1 = (dot(P.d[0], disp) > 0) ? 1.0 : 0.0;
    return w0 * v0_phase + w1 * ph1;
  }
  const V3& v2 = P.v[1];
  const V3& v3 = P.v[2];
  const V3 a1 = v1 - v0, a2 = v2 - v0, a3 = v3 - v0;
  const double o012 = std::abs(dot(cross(a1, a2), v0));
  const double o013 = std::abs(dot(cross(a1, a3), v0));
  const double o023 = std::abs(dot(cross(a2, a3), v0));
  const double o123 = std::abs(dot(cross(v2 - v1, v3 - v1), v1));
  const double vol = ((o012 + o013) + o023) + o123;
  if (vol <= 0.0) return 0.0;
  const double inv = 1.0 / vol;
  const double w0 = o123 * inv, w1 = o023 * inv, w2 = o013 * inv, w3 = o012 * inv;
  const double ph1 = (dot(P.d[0], disp) > 0) ? 1.0 : 0.0;
  const double ph2 = (dot(P.d[1], disp) > 0) ? 1.0 : 0.0;
  const double ph3 = (dot(P.d[2], disp) > 0) ? 1.0 : 0.0;
  return ((w0 * v0_phase + w1 * ph1) + w2 * ph2) + w3 * ph3;
}

// Local AABB of a shape (computeLocalAABB; a hull's from its vertices,
// convex-inl.h:76-87): lo, hi.
inline void localAabb(const Shape& s, double lo[3], double hi[3]) {
  switch (s.type) {
    case kBox: for (int k = 0; k < 3; ++k) hi[k] = 0.5 * s.p[k]; break;
    case kSphere: hi[0] = hi[1] = hi[2] = s.p[0]; break;
    case kCapsule: hi[0] = hi[1] = s.p[0]; hi[2] = 0.5 * s.p[1] + s.p[0]; break;
    case kCylinder: hi[0] = hi[1] = s.p[0]; hi[2] = 0.5 * s.p[1]; break;
    default: {
      for (int k = 0; k < 3; ++k) { lo[k] = 1e300; hi[k] = -1e300; }
      for (int v = 0; v < s.nv; ++v)
        for (int k = 0; k < 3; ++k) {
          const double x = s.verts[4 * (size_t)v + k];
          lo[k] = std::min(lo[k], x);
          hi[k] = std::max(hi[k], x);
        }
      return;
    }
  }
  for (int k = 0; k < 3; ++k) lo[k] = -hi[k];
}

struct CcdOut {
  bool collide = false;
  Interval toc;           // (-1, -1) when the request computes none
  int mpr_status = -1;    // MPRStatus of the swept-volume run, -1 when none ran
  bool box_tested = false;
};

// The boxes of a pair as the approximate request builds them (convertBV of
// each shape's local AABB, utility-inl.h:586-607; computeBV<OBB> for a box,
// geometry/shape/utility-inl.h:93-99) and BoxPairTranslationalCCD::IsDisjoint
// (box_pair_ccd-inl.h:365-393): box 1 in its own frame, box 2 by the pose.
inline bool obbPairDisjoint(const Shape& a, const Shape& b, const Iso& pose, const V3& axis, double dist,
                            double zero_tol, Interval& iv) {
  double lo1[3], hi1[3], lo2[3], hi2[3];
  localAabb(a, lo1, hi1);
  localAabb(b, lo2, hi2);
  double h1[3], h2[3];
  V3 c1, c2;
  for (int k = 0; k < 3; ++k) {
    h1[k] = (hi1[k] - lo1[k]) * 0.5;
    h2[k] = (hi2[k] - lo2[k]) * 0.5;
    c1[k] = (lo1[k] + hi1[k]) * 0.5;
    c2[k] = (lo2[k] + hi2[k]) * 0.5;
  }
  if (a.type == kBox) c1 = V3(0, 0, 0);
  if (b.type == kBox) c2 = V3(0, 0, 0);
  // box 2's centre in box 1's frame: pose * c2 - c1 (box 1's axes are its frame's)
  const V3 To2(((pose.R[0] * c2.x + pose.R[1] * c2.y) + pose.R[2] * c2.z) + pose.t.x,
               ((pose.R[3] * c2.x + pose.R[4] * c2.y) + pose.R[5] * c2.z) + pose.t.y,
               ((pose.R[6] * c2.x + pose.R[7] * c2.y) + pose.R[8] * c2.z) + pose.t.z);
  const V3 t = To2 - c1;
  return boxPairDisjoint(h1, axis, dist, pose.R, t, h2, zero_tol, iv);
}

// One shape pair (ShapePairTranslationalCollisionImpl::RunIntersect,
// shape_pair_ccd-inl.h:57-150): box-box pairs take the box interval alone
// (:113-133); other pairs by request type.
inline CcdOut translationalCcd(const Shape& a, const Shape& b, const Iso& pose, const V3& axis, double dist,
                               TocRequest req, double zero_tol, int max_iter, double tol) {
  CcdOut o;
  if (a.type == kBox && b.type == kBox) {
    Interval iv;
    o.box_tested = true;
    o.collide = !obbPairDisjoint(a, b, pose, axis, dist, zero_tol, iv);
    if (o.collide) o.toc = iv;
    return o;
  }
  if (req == TocRequest::BoxApproximate) {
    Interval iv;
    o.box_tested = true;
    if (obbPairDisjoint(a, b, pose, axis, dist, zero_tol, iv)) return o;
    o.toc = iv;
  }
  MinkDiff md;
  md.s0 = &a;
  md.s1 = &b;
  md.to0 = pose;
  md.swept = true;
  md.sweep = axis * dist;
  MPR mpr(max_iter, tol);
  MPRPortal P;
  const MPRStatus ms = mpr.Intersect(md, &P);
  o.mpr_status = (int)ms;
  o.collide = ms == MPRStatus::Intersect;
  if (!o.collide) {
    o.toc = Interval();
    return o;
  }
  if (req == TocRequest::OneTocSample) {
    const double ts = tocSample(md.sweep, P);
    o.toc.lo = o.toc.hi = ts;
  }
  return o;
}

}  // namespace orc
