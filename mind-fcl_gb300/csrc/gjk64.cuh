// GJK boolean + GJK separation distance in FP64, one thread per pair: the
// plain method the FP32 kernels (gjk.cuh) approximate, with the reference's
// FP64 arithmetic (cvx_collide/gjk.hpp:10-363, gjk_distance.hpp:10-559).
// The control flow is gjk.cuh's, branch for branch; here every quantity is
// FP64 and every arithmetic operation rounds on its own (no fused
// multiply-add), as the reference's scalar code, so the flags, statuses and
// witness points follow the reference to FP64 rounding.  Supports restate
// gjk_shape.hpp:40-180 and the convex scan convex-inl.h:133-149 on the FP32
// inputs promoted to FP64.
//
// nvcc builds it for the device.  Defining FCLG64_HOST (after declaring
// ShapeDev, float4 and the shape and GJK status codes of device_math.cuh)
// builds the same functions for the CPU, where, compiled without contraction
// (-ffp-contract=off), every operation rounds as on the device: the tests
// check that build against the reference's outputs bit for bit.
#pragma once
#ifndef FCLG64_HOST
#include "device_math.cuh"
#define FCLG64_FN __device__ __forceinline__
#define FCLG64_COLD __device__
#define FCLG64_LDG(p) __ldg(p)
#else
#include <cmath>
#define FCLG64_FN inline
#define FCLG64_COLD inline
#define FCLG64_LDG(p) (*(p))
#endif

namespace fclg {
namespace f64 {

#ifndef FCLG64_HOST
FCLG64_FN double dmul(double a, double b) { return __dmul_rn(a, b); }
FCLG64_FN double dadd(double a, double b) { return __dadd_rn(a, b); }
FCLG64_FN double dsub(double a, double b) { return __dsub_rn(a, b); }
FCLG64_FN double ddiv(double a, double b) { return __ddiv_rn(a, b); }
FCLG64_FN double dsqrt(double a) { return __dsqrt_rn(a); }
#else
FCLG64_FN double dmul(double a, double b) { return a * b; }
FCLG64_FN double dadd(double a, double b) { return a + b; }
FCLG64_FN double dsub(double a, double b) { return a - b; }
FCLG64_FN double ddiv(double a, double b) { return a / b; }
FCLG64_FN double dsqrt(double a) { return std::sqrt(a); }
#endif

struct v3 {
  double x, y, z;
};
FCLG64_FN v3 mk3(double x, double y, double z) { return v3{x, y, z}; }
FCLG64_FN v3 operator+(v3 a, v3 b) { return v3{dadd(a.x, b.x), dadd(a.y, b.y), dadd(a.z, b.z)}; }
FCLG64_FN v3 operator-(v3 a, v3 b) { return v3{dsub(a.x, b.x), dsub(a.y, b.y), dsub(a.z, b.z)}; }
FCLG64_FN v3 operator-(v3 a) { return v3{-a.x, -a.y, -a.z}; }
FCLG64_FN v3 operator*(v3 a, double s) { return v3{dmul(a.x, s), dmul(a.y, s), dmul(a.z, s)}; }
FCLG64_FN v3 operator*(double s, v3 a) { return v3{dmul(s, a.x), dmul(s, a.y), dmul(s, a.z)}; }
FCLG64_FN double dot(v3 a, v3 b) { return dadd(dadd(dmul(a.x, b.x), dmul(a.y, b.y)), dmul(a.z, b.z)); }
FCLG64_FN v3 cross(v3 a, v3 b) {
  return v3{dsub(dmul(a.y, b.z), dmul(a.z, b.y)), dsub(dmul(a.z, b.x), dmul(a.x, b.z)),
            dsub(dmul(a.x, b.y), dmul(a.y, b.x))};
}
FCLG64_FN double sqn(v3 a) { return dot(a, a); }
FCLG64_FN double nrm(v3 a) { return dsqrt(sqn(a)); }
// divides each coefficient by the norm; leaves a zero vector unchanged
FCLG64_FN v3 normalized(v3 a) {
  const double n2 = sqn(a);
  if (!(n2 > 0.)) return a;
  const double n = dsqrt(n2);
  return v3{ddiv(a.x, n), ddiv(a.y, n), ddiv(a.z, n)};
}

// Pose of shape b in shape a's frame (FP32 input promoted to FP64).
struct Pose64 {
  double r[9];
  v3 t;
  FCLG64_FN v3 rot(v3 v) const {
    return v3{dadd(dadd(dmul(r[0], v.x), dmul(r[1], v.y)), dmul(r[2], v.z)),
              dadd(dadd(dmul(r[3], v.x), dmul(r[4], v.y)), dmul(r[5], v.z)),
              dadd(dadd(dmul(r[6], v.x), dmul(r[7], v.y)), dmul(r[8], v.z))};
  }
  FCLG64_FN v3 rotT(v3 v) const {
    return v3{dadd(dadd(dmul(r[0], v.x), dmul(r[3], v.y)), dmul(r[6], v.z)),
              dadd(dadd(dmul(r[1], v.x), dmul(r[4], v.y)), dmul(r[7], v.z)),
              dadd(dadd(dmul(r[2], v.x), dmul(r[5], v.y)), dmul(r[8], v.z))};
  }
  FCLG64_FN v3 apply(v3 v) const { return rot(v) + t; }
};

// gjk_shape.hpp:40-180 (box full side stored, half used; capsule / cylinder
// half length) and the convex naive scan (first maximum), convex-inl.h:133-149.
FCLG64_FN v3 shape_support(const ShapeDev& s, const float4* __restrict__ verts, v3 d) {
  switch (s.type) {
    case kBox:
      return v3{d.x > 0. ? (double)s.p0 : -(double)s.p0, d.y > 0. ? (double)s.p1 : -(double)s.p1,
                d.z > 0. ? (double)s.p2 : -(double)s.p2};
    case kSphere:
      return d * (double)s.p0;
    case kCapsule: {
      const v3 v = d * (double)s.p0;
      const v3 pos1 = v3{dadd(0., v.x), dadd(0., v.y), dadd((double)s.p1, v.z)};
      const v3 pos2 = v3{dadd(0., v.x), dadd(0., v.y), dadd(-(double)s.p1, v.z)};
      return dot(d, pos1) > dot(d, pos2) ? pos1 : pos2;
    }
    case kCylinder: {
      const double zdist = dsqrt(dadd(dmul(d.x, d.x), dmul(d.y, d.y)));
      const double z = d.z > 0. ? (double)s.p1 : -(double)s.p1;
      if (zdist == 0.) return v3{0., 0., z};
      const double k = ddiv((double)s.p0, zdist);
      return v3{dmul(k, d.x), dmul(k, d.y), z};
    }
    case kConvex: {
      const float4* v = verts + s.vofs;
      uint32_t best_i = 0;
      double best = -1.;
      for (uint32_t i = 0; i < s.nv; ++i) {
        const float4 q = FCLG64_LDG(v + i);
        const double val = dot(d, v3{q.x, q.y, q.z});
        if (i == 0 || val > best) {
          best = val;
          best_i = i;
        }
      }
      const float4 q = FCLG64_LDG(v + best_i);
      return v3{q.x, q.y, q.z};
    }
    default:
      return v3{0., 0., 0.};
  }
}

// Support of A - B with B posed in A's frame (minkowski_diff.hpp:21-58).
struct MinkowskiSupport64 {
  ShapeDev A, B;
  Pose64 pose;
  const float4* __restrict__ verts;
  FCLG64_FN void operator()(v3 d, v3& pa, v3& pb) const {
    pa = shape_support(A, verts, d);
    pb = pose.apply(shape_support(B, verts, pose.rotT(-d)));
  }
};

struct Simplex {
  v3 w[4];   // Minkowski-difference vertex = a - b
  v3 a[4];   // support point on shape a (a's frame)
  v3 b[4];   // support point on shape b (a's frame)
  int rank;
  FCLG64_FN void set(int i, v3 pa, v3 pb) {
    a[i] = pa;
    b[i] = pb;
    w[i] = pa - pb;
  }
  FCLG64_FN void copy(int dst, int src) {
    w[dst] = w[src];
    a[dst] = a[src];
    b[dst] = b[src];
  }
};

enum class Proj { Failed, Continue, Intersect, ZeroVolume };
enum class Upd { NoImprovement, OK, Failed };

struct GjkOut {
  int status;      // GJK_Status
  bool point_valid;
  v3 p0, p1;       // witness points (a's frame) when separated
  int iterations;  // boolean + distance loop iterations
};

// gjk.hpp:161-197
FCLG64_FN Proj project2(Simplex& s, v3& d) {
  const v3 a = s.w[1], b = s.w[0];
  const v3 a_to_b = b - a;
  const double ao_dot_ab = -dot(a_to_b, a);
  const v3 ab_cross_ao = cross(a, a_to_b);
  if (ao_dot_ab > 0. && sqn(ab_cross_ao) <= 0.) return Proj::Intersect;
  if (ao_dot_ab <= 0.) {
    s.copy(0, 1);
    s.rank = 1;
    d = -normalized(a);
    return Proj::Continue;
  }
  d = normalized(cross(ab_cross_ao, a_to_b));
  return Proj::Continue;
}

// gjk.hpp:199-278
FCLG64_FN Proj project3(Simplex& s, v3& d, double tol) {
  const v3 a = s.w[2], b = s.w[1], c = s.w[0];
  const v3 a_to_b = b - a, a_to_c = c - a;
  const bool sep_b = dot(a, a_to_b) >= 0.;
  const bool sep_c = dot(a, a_to_c) >= 0.;
  if (sep_b && sep_c) {
    s.copy(0, 2);
    s.rank = 1;
    d = normalized(-a);
    return Proj::Continue;
  }
  const v3 n = cross(a_to_b, a_to_c);
  const v3 ac_normal = cross(n, a_to_c);
  if (dot(a, ac_normal) <= 0.) {
    s.copy(1, 2);
    s.rank = 2;
    d = normalized(cross(cross(a, a_to_c), a_to_c));
    return Proj::Continue;
  }
  const v3 ab_normal = cross(a_to_b, n);
  if (dot(a, ab_normal) <= 0.) {
    s.copy(0, 1);
    s.copy(1, 2);
    s.rank = 2;
    d = normalized(cross(cross(a, a_to_b), a_to_b));
    return Proj::Continue;
  }
  const double area = nrm(n);
  if (area < tol * tol) return Proj::Failed;
  const v3 nu = v3{ddiv(n.x, area), ddiv(n.y, area), ddiv(n.z, area)};
  const double nu_dot_a = dot(nu, a);
  if (fabs(nu_dot_a) < tol) return Proj::Intersect;
  d = (nu_dot_a <= 0.) ? nu : -nu;
  return Proj::Continue;
}

// gjk.hpp:280-360
FCLG64_COLD Proj project4(Simplex& s, v3& dir, double tol) {
  const v3 a = s.w[3], b = s.w[2], c = s.w[1], dd = s.w[0];
  const v3 ab = b - a, ac = c - a, ad = dd - a;
  v3 abc = cross(ab, ac), acd = cross(ac, ad), abd = cross(ab, ad);
  const double abc_ad = dot(abc, ad), acd_ab = dot(acd, ab), abd_ac = dot(abd, ac);
  if (fabs(abc_ad) <= 0.0) return Proj::ZeroVolume;
  if (abc_ad > 0) abc = abc * -1.0;
  if (acd_ab > 0) acd = acd * -1.0;
  if (abd_ac > 0) abd = abd * -1.0;
  const bool d_side = dot(a, abc) > 0;
  const bool c_side = dot(a, abd) > 0;
  const bool b_side = dot(a, acd) > 0;
  if (d_side && c_side && b_side) return Proj::Intersect;
  if (!b_side) {
    s.copy(2, 3);
  } else if (!c_side) {
    s.copy(1, 2);
    s.copy(2, 3);
  } else {
    s.copy(0, 1);
    s.copy(1, 2);
    s.copy(2, 3);
  }
  s.rank = 3;
  return project3(s, dir, tol);
}

// gjk_distance.hpp:128-153 (on simplex slots 1 = newest, 0)
FCLG64_FN void update2(Simplex& s, v3& out, double tol) {
  const v3 s1 = s.w[1], s2 = s.w[0];
  const v3 s1_to_s2 = s2 - s1;
  const double len2 = sqn(s1_to_s2);
  const double t = -dot(s1, s1_to_s2);
  if (t <= 0. || len2 <= tol * tol) {
    out = s1;
    s.copy(0, 1);
    s.rank = 1;
  } else if (t >= len2) {
    out = s2;
    s.rank = 1;
  } else {
    const double w2 = t / len2;
    out = w2 * s2 + (1. - w2) * s1;
  }
}

// gjk_distance.hpp:155-286 (slot 2 newest)
FCLG64_FN void update3(Simplex& s, v3& out, double tol) {
  const v3 s1 = s.w[2], s2 = s.w[1], s3 = s.w[0];
  const v3 s1_to_s2 = s2 - s1, s1_to_s3 = s3 - s1;
  const bool sep2 = dot(s1, s1_to_s2) >= 0.;
  const bool sep3 = dot(s1, s1_to_s3) >= 0.;
  if (sep2 && sep3) {
    out = s1;
    s.copy(0, 2);
    s.rank = 1;
    return;
  }
  const v3 n = cross(s1_to_s2, s1_to_s3);
  const double area2 = sqn(n);
  const bool zero_area = area2 <= 0.;
  const bool s12_sep = dot(s1, cross(n, s1_to_s2)) > 0.;
  if (!sep2 && s12_sep) {
    s.copy(0, 1);
    s.copy(1, 2);
    s.rank = 2;
    update2(s, out, tol);
    return;
  }
  const bool s13_sep = dot(s1, cross(n, s1_to_s3)) < 0.;
  if (!sep3 && s13_sep) {
    s.copy(1, 2);
    s.rank = 2;
    update2(s, out, tol);
    return;
  }
  double best = -1.;
  v3 best_pt = mk3(0, 0, 0), pt;
  Simplex best_s = s, c;
  if (zero_area || s12_sep) {
    c = s;
    c.copy(0, 1);
    c.copy(1, 2);
    c.rank = 2;
    update2(c, pt, tol);
    const double dd = sqn(pt);
    if (best < 0. || dd < best) { best = dd; best_s = c; best_pt = pt; }
  }
  if (zero_area || s13_sep) {
    c = s;
    c.copy(1, 2);
    c.rank = 2;
    update2(c, pt, tol);
    const double dd = sqn(pt);
    if (best < 0. || dd < best) { best = dd; best_s = c; best_pt = pt; }
  }
  const bool s23_sep = dot(s2, cross(n, s3 - s2)) > 0.;
  if (zero_area || s23_sep) {
    c = s;
    c.rank = 2;
    update2(c, pt, tol);
    const double dd = sqn(pt);
    if (best < 0. || dd < best) { best = dd; best_s = c; best_pt = pt; }
  }
  if (best < 0.) {
    out = n * (dot(s1, n) / area2);
  } else {
    s = best_s;
    out = best_pt;
  }
}

// gjk_distance.hpp:288-373 (slot 3 newest): best of faces (3,2,1), (3,2,0), (3,1,0).
FCLG64_COLD Upd update4(Simplex& s, v3& out, double tol) {
  double best = -1.;
  v3 best_pt = mk3(0, 0, 0), pt;
  Simplex best_s = s, c;
  c = s;
  c.copy(0, 1); c.copy(1, 2); c.copy(2, 3);
  c.rank = 3;
  update3(c, pt, tol);
  double dd = sqn(pt);
  if (best < 0. || dd < best) { best = dd; best_pt = pt; best_s = c; }
  c = s;
  c.copy(1, 2); c.copy(2, 3);
  c.rank = 3;
  update3(c, pt, tol);
  dd = sqn(pt);
  if (best < 0. || dd < best) { best = dd; best_pt = pt; best_s = c; }
  c = s;
  c.copy(2, 3);
  c.rank = 3;
  update3(c, pt, tol);
  dd = sqn(pt);
  if (best < 0. || dd < best) { best = dd; best_pt = pt; best_s = c; }
  if (best < 0.) return Upd::NoImprovement;
  s = best_s;
  out = best_pt;
  return Upd::OK;
}

FCLG64_FN Upd update_simplex(Simplex& s, v3& out, double tol) {
  if (s.rank == 1) { out = s.w[0]; return Upd::OK; }
  if (s.rank == 2) { update2(s, out, tol); return Upd::OK; }
  if (s.rank == 3) { update3(s, out, tol); return Upd::OK; }
  if (s.rank == 4) return update4(s, out, tol);
  return Upd::Failed;
}

// gjk_distance.hpp:375-470; the stored support points replace the
// reference's re-evaluation of support0/support1 at the stored directions.
FCLG64_COLD bool extract_no_sub(const Simplex& s, v3& p0, v3& p1) {
  constexpr double kBaryTol = 1e-3;
  if (s.rank == 4 || s.rank < 1) return false;
  if (s.rank == 1) {
    p0 = s.a[0];
    p1 = s.b[0];
    return true;
  }
  if (s.rank == 2) {
    const v3 s1_to_s2 = s.w[1] - s.w[0];
    const double len2 = sqn(s1_to_s2);
    if (len2 <= 0.) {
      p0 = s.a[0];
      p1 = s.b[0];
      return true;
    }
    const double w2 = -dot(s.w[0], s1_to_s2) / len2;
    if (w2 > 1. + kBaryTol) { p0 = s.a[1]; p1 = s.b[1]; return false; }
    if (w2 < -kBaryTol) { p0 = s.a[0]; p1 = s.b[0]; return false; }
    const double w1 = 1. - w2;
    p0 = s.a[0] * w1 + s.a[1] * w2;
    p1 = s.b[0] * w1 + s.b[1] * w2;
    return true;
  }
  // triangle: barycentric weights from areas, each within the tolerance of [0, 1]
  const v3 s1_to_s2 = s.w[1] - s.w[0], s1_to_s3 = s.w[2] - s.w[0];
  const v3 n = cross(s1_to_s2, s1_to_s3);
  const double area2 = sqn(n);
  if (area2 <= 0.) return false;
  const v3 proj = n * ddiv(dot(s.w[0], n), area2);
  const double area = dsqrt(area2);
  const double w2 = ddiv(nrm(cross(s1_to_s3, s.w[0] - proj)), area);
  const double w3 = ddiv(nrm(cross(s1_to_s2, s.w[0] - proj)), area);
  const double w1 = dsub(dsub(1., w2), w3);
  if (w1 < -kBaryTol || w2 < -kBaryTol || w3 < -kBaryTol) return false;
  p0 = (s.a[0] * w1 + s.a[1] * w2) + s.a[2] * w3;
  p1 = (s.b[0] * w1 + s.b[1] * w2) + s.b[2] * w3;
  return true;
}

// gjk_distance.hpp:472-559
FCLG64_COLD bool extract_try_sub(const Simplex& s, v3& p0, v3& p1) {
  if (s.rank >= 4) return false;
  if (s.rank <= 2) {
    extract_no_sub(s, p0, p1);
    return true;
  }
  double best = -1.;
  v3 b0 = mk3(0, 0, 0), b1 = mk3(0, 0, 0), c0, c1;
  Simplex c = s;
  if (extract_no_sub(c, c0, c1)) {
    const double dd = sqn(c0 - c1);
    if (best < 0. || dd < best) { best = dd; b0 = c0; b1 = c1; }
  }
  c = s;
  c.rank = 2;
  extract_no_sub(c, c0, c1);
  double dd = sqn(c0 - c1);
  if (best < 0. || dd < best) { best = dd; b0 = c0; b1 = c1; }
  c = s;
  c.copy(1, 2);
  c.rank = 2;
  extract_no_sub(c, c0, c1);
  dd = sqn(c0 - c1);
  if (best < 0. || dd < best) { best = dd; b0 = c0; b1 = c1; }
  c = s;
  c.copy(0, 1);
  c.copy(1, 2);
  c.rank = 2;
  extract_no_sub(c, c0, c1);
  dd = sqn(c0 - c1);
  if (best < 0. || dd < best) { best = dd; b0 = c0; b1 = c1; }
  p0 = b0;
  p1 = b1;
  return true;
}

// gjk_distance.hpp:10-105: minimum distance from a separating vertex.
template <class Sup>
FCLG64_FN bool min_distance(const Sup& sup, Simplex& s, double tol, int max_iter, v3& p0, v3& p1,
                                             int& iters) {
  v3 cur;
  if (update_simplex(s, cur, tol) != Upd::OK) return false;
  double book = nrm(cur);
  if (book <= tol) return extract_no_sub(s, p0, p1);
  v3 next = v3{ddiv(-cur.x, book), ddiv(-cur.y, book), ddiv(-cur.z, book)};
  const double tol2 = tol * tol;
  for (int it = 0; it < max_iter; ++it) {
    ++iters;
    v3 pa, pb;
    sup(next, pa, pb);
    const v3 w = pa - pb;
    if (dot(next, w - cur) < tol) return extract_no_sub(s, p0, p1);
    bool dup = false;
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (j < s.rank && sqn(s.w[j] - w) < tol2) dup = true;
    if (dup) return extract_no_sub(s, p0, p1);
    // s.rank is 1..3 here
    if (s.rank == 1) s.set(1, pa, pb);
    else if (s.rank == 2) s.set(2, pa, pb);
    else s.set(3, pa, pb);
    s.rank += 1;
    const Upd st = update_simplex(s, cur, tol);
    if (st == Upd::NoImprovement) return extract_no_sub(s, p0, p1);
    if (st != Upd::OK) return false;
    const double nd = nrm(cur);
    if (book - nd < tol) return extract_no_sub(s, p0, p1);
    if (nd < tol) return extract_no_sub(s, p0, p1);
    book = nd;
    next = v3{ddiv(-cur.x, book), ddiv(-cur.y, book), ddiv(-cur.z, book)};
  }
  return false;
}

// gjk.hpp:10-140.  want_distance selects the MinSeparationDistanceOutput path.
template <class Sup>
FCLG64_FN GjkOut gjk_evaluate(const Sup& sup, v3 guess, double tol, int max_iter, bool want_distance,
                                               Simplex& s) {
  GjkOut o;
  o.point_valid = false;
  o.iterations = 0;
  o.p0 = o.p1 = mk3(0, 0, 0);
  v3 d = guess;
  if (sqn(d) <= 0.) d = mk3(1, 0, 0);
  d = normalized(d);
  const double tol2 = tol * tol;
  v3 pa, pb;
  sup(d, pa, pb);
  s.set(0, pa, pb);
  s.rank = 1;
  if (sqn(s.w[0]) <= tol2) { o.status = kGjkIntersect; return o; }
  bool separated = dot(s.w[0], d) < 0.;
  int undetermined = -1;
  if (!separated) {
    d = -d;
    int it = 0;
    for (; it < max_iter; ++it) {
      o.iterations = it + 1;
      sup(d, pa, pb);
      const v3 w = pa - pb;
      if (dot(w, d) < 0.) {
        s.set(0, pa, pb);  // the separating vertex seeds the distance simplex
        s.rank = 1;
        separated = true;
        break;
      }
      bool dup = false;
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (j < s.rank && sqn(s.w[j] - w) < tol2) dup = true;
      if (dup) { undetermined = kGjkNoProgress; break; }
      if (s.rank == 1) s.set(1, pa, pb);
      else if (s.rank == 2) s.set(2, pa, pb);
      else s.set(3, pa, pb);
      s.rank += 1;
      if (sqn(w) <= tol2) { o.status = kGjkIntersect; return o; }
      Proj st;
      if (s.rank == 2) st = project2(s, d);
      else if (s.rank == 3) st = project3(s, d, tol);
      else st = project4(s, d, tol);
      if (st == Proj::Failed) { o.status = kGjkFailed; return o; }
      if (st == Proj::Intersect) { o.status = kGjkIntersect; return o; }
      if (st == Proj::ZeroVolume) { undetermined = kGjkNoProgress; break; }
    }
    if (!separated && undetermined < 0) undetermined = kGjkIterLimit;
  } else {
    s.rank = 1;
  }
  if (separated) {
    o.status = kGjkSeparated;
    if (want_distance) o.point_valid = min_distance(sup, s, tol, max_iter, o.p0, o.p1, o.iterations);
    return o;
  }
  o.status = undetermined;
  if (want_distance) o.point_valid = extract_try_sub(s, o.p0, o.p1);
  return o;
}


}  // namespace f64
}  // namespace fclg
