// GJK boolean + GJK separation distance in FP32, one pair per group of LANES
// lanes.  The control flow restates the reference's GJK (gjk.hpp:10-363) and
// its minimum-distance loop (gjk_distance.hpp:10-559) branch for branch, so
// that the flag, the status and the witness points agree with the FP64
// reference except where FP32 rounding moves a decision that sits within a
// few ulps of its threshold.  The tetrahedron orientation tests of
// simplexProjection4 (the degenerate-simplex determinants) run in FP64.
//
// All lanes of a group run this scalar code redundantly on identical values;
// only the support evaluations split work across the group.
#pragma once
#include "support.cuh"

#ifndef FCLG_GJK_TRACE
#define FCLG_GJK_TRACE(...) \
  do {                      \
  } while (0)
#endif

// Inline policy of the simplex routines that run at most once per pair or
// only at rank 4 (kept out of line by a build that defines
// FCLG_GJK_COLD_OUTLINED, or FCLG_GJK_COLD itself).
#ifndef FCLG_GJK_COLD
#ifdef FCLG_GJK_COLD_OUTLINED
#define FCLG_GJK_COLD static __noinline__
#else
#define FCLG_GJK_COLD __forceinline__
#endif
#endif

namespace fclg {

struct Simplex {
  f3 w[4];   // Minkowski-difference vertex = a - b
  f3 a[4];   // support point on shape a (a's frame)
  f3 b[4];   // support point on shape b (a's frame)
  int rank;
  __device__ __forceinline__ void set(int i, f3 pa, f3 pb) {
    a[i] = pa;
    b[i] = pb;
    w[i] = pa - pb;
  }
  __device__ __forceinline__ void copy(int dst, int src) {
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
  f3 p0, p1;       // witness points (a's frame) when separated
  int iterations;  // boolean + distance loop iterations
};

// gjk.hpp:161-197
__device__ __forceinline__ Proj project2(Simplex& s, f3& d) {
  const f3 a = s.w[1], b = s.w[0];
  const f3 a_to_b = b - a;
  const float ao_dot_ab = -dot(a_to_b, a);
  const f3 ab_cross_ao = cross(a, a_to_b);
  if (ao_dot_ab > 0.f && sqn(ab_cross_ao) <= 0.f) return Proj::Intersect;
  if (ao_dot_ab <= 0.f) {
    s.copy(0, 1);
    s.rank = 1;
    d = -normalized(a);
    return Proj::Continue;
  }
  d = normalized(cross(ab_cross_ao, a_to_b));
  return Proj::Continue;
}

// gjk.hpp:199-278
__device__ __forceinline__ Proj project3(Simplex& s, f3& d, float tol) {
  const f3 a = s.w[2], b = s.w[1], c = s.w[0];
  const f3 a_to_b = b - a, a_to_c = c - a;
  const bool sep_b = dot(a, a_to_b) >= 0.f;
  const bool sep_c = dot(a, a_to_c) >= 0.f;
  if (sep_b && sep_c) {
    s.copy(0, 2);
    s.rank = 1;
    d = normalized(-a);
    return Proj::Continue;
  }
  const f3 n = cross(a_to_b, a_to_c);
  const f3 ac_normal = cross(n, a_to_c);
  if (dot(a, ac_normal) <= 0.f) {
    s.copy(1, 2);
    s.rank = 2;
    d = normalized(cross(cross(a, a_to_c), a_to_c));
    return Proj::Continue;
  }
  const f3 ab_normal = cross(a_to_b, n);
  if (dot(a, ab_normal) <= 0.f) {
    s.copy(0, 1);
    s.copy(1, 2);
    s.rank = 2;
    d = normalized(cross(cross(a, a_to_b), a_to_b));
    return Proj::Continue;
  }
  const float area = nrm(n);
  if (area < tol * tol) return Proj::Failed;
  const f3 nu = n * (1.f / area);
  const float nu_dot_a = dot(nu, a);
  if (fabsf(nu_dot_a) < tol) return Proj::Intersect;
  d = (nu_dot_a <= 0.f) ? nu : -nu;
  return Proj::Continue;
}

// Triple product u . (v x w) in FP32 with a bound on its error: the inputs are
// differences of FP32 points rounded once (or exact), so the computed value is
// within 8 eps of |u| . (|v| x+ |w|) of the exact one (eps = 2^-24; the bound
// below keeps a factor of four in hand).  certain: the sign is the exact one.
__device__ __forceinline__ float triple_filtered(f3 u, f3 v, f3 w, bool& certain) {
  const float t = dot(u, cross(v, w));
  const f3 au = mk3(fabsf(u.x), fabsf(u.y), fabsf(u.z));
  const f3 av = mk3(fabsf(v.x), fabsf(v.y), fabsf(v.z));
  const f3 aw = mk3(fabsf(w.x), fabsf(w.y), fabsf(w.z));
  const float mag = au.x * (av.y * aw.z + av.z * aw.y) + au.y * (av.z * aw.x + av.x * aw.z) +
                    au.z * (av.x * aw.y + av.y * aw.x);
  // 32 * 2^-24; below 1e-30 the products may be subnormal: no certainty
  certain = certain && mag > 1e-30f && fabsf(t) > 1.9073486e-06f * mag;
  return t;
}

// gjk.hpp:280-360.  The orientation tests decide the branch by their signs
// alone: they run in FP32 with an error bound (triple_filtered) and again in
// FP64 only when a sign is within the bound (near-degenerate tetrahedra), so
// the decisions are the FP64 tests' everywhere.
__device__ FCLG_GJK_COLD Proj project4(Simplex& s, f3& dir, float tol) {
  bool zero_volume, d_side, c_side, b_side;
  {
    const f3 a = s.w[3], b = s.w[2], c = s.w[1], dd = s.w[0];
    const f3 ab = b - a, ac = c - a, ad = dd - a;
    bool certain = true;
    // abc . ad = ad . (ab x ac), acd . ab = ab . (ac x ad), abd . ac = ac . (ab x ad)
    const float abc_ad = triple_filtered(ad, ab, ac, certain);
    const float acd_ab = triple_filtered(ab, ac, ad, certain);
    const float abd_ac = triple_filtered(ac, ab, ad, certain);
    // the side tests a . n with each normal turned away from the fourth vertex
    const float sd = triple_filtered(a, ab, ac, certain);
    const float sc = triple_filtered(a, ab, ad, certain);
    const float sb = triple_filtered(a, ac, ad, certain);
    zero_volume = false;
    d_side = abc_ad > 0.f ? sd < 0.f : sd > 0.f;
    c_side = abd_ac > 0.f ? sc < 0.f : sc > 0.f;
    b_side = acd_ab > 0.f ? sb < 0.f : sb > 0.f;
    if (!certain) {
      const d3 a = tod(s.w[3]), b = tod(s.w[2]), c = tod(s.w[1]), dd = tod(s.w[0]);
      const d3 ab = b - a, ac = c - a, ad = dd - a;
      d3 abc = cross(ab, ac), acd = cross(ac, ad), abd = cross(ab, ad);
      const double abc_ad = dot(abc, ad), acd_ab = dot(acd, ab), abd_ac = dot(abd, ac);
      zero_volume = fabs(abc_ad) <= 0.0;
      if (abc_ad > 0) abc = abc * -1.0;
      if (acd_ab > 0) acd = acd * -1.0;
      if (abd_ac > 0) abd = abd * -1.0;
      d_side = dot(a, abc) > 0;
      c_side = dot(a, abd) > 0;
      b_side = dot(a, acd) > 0;
    }
  }
  if (zero_volume) return Proj::ZeroVolume;
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
__device__ __forceinline__ void update2(Simplex& s, f3& out, float tol) {
  const f3 s1 = s.w[1], s2 = s.w[0];
  const f3 s1_to_s2 = s2 - s1;
  const float len2 = sqn(s1_to_s2);
  const float t = -dot(s1, s1_to_s2);
  if (t <= 0.f || len2 <= tol * tol) {
    out = s1;
    s.copy(0, 1);
    s.rank = 1;
  } else if (t >= len2) {
    out = s2;
    s.rank = 1;
  } else {
    const float w2 = t / len2;
    out = w2 * s2 + (1.f - w2) * s1;
  }
}

// gjk_distance.hpp:155-286 (slot 2 newest).  The segment candidates --
// (s2, s1), (s3, s1), (s3, s2), in that order, the first of equal distances
// kept -- run through one update2 call site in a loop, so the routine holds a
// single copy of update2's code.
__device__ __forceinline__ void update3(Simplex& s, f3& out, float tol) {
  const f3 s1 = s.w[2], s2 = s.w[1], s3 = s.w[0];
  const f3 s1_to_s2 = s2 - s1, s1_to_s3 = s3 - s1;
  const bool sep2 = dot(s1, s1_to_s2) >= 0.f;
  const bool sep3 = dot(s1, s1_to_s3) >= 0.f;
  if (sep2 && sep3) {
    out = s1;
    s.copy(0, 2);
    s.rank = 1;
    return;
  }
  const f3 n = cross(s1_to_s2, s1_to_s3);
  const float area2 = sqn(n);
  const bool zero_area = area2 <= 0.f;
  const bool s12_sep = dot(s1, cross(n, s1_to_s2)) > 0.f;
  unsigned cand;
  if (!sep2 && s12_sep) {
    cand = 1u;  // segment s1 s2 alone
  } else {
    const bool s13_sep = dot(s1, cross(n, s1_to_s3)) < 0.f;
    if (!sep3 && s13_sep) {
      cand = 2u;  // segment s1 s3 alone
    } else {
      const bool s23_sep = dot(s2, cross(n, s3 - s2)) > 0.f;
      cand = ((zero_area || s12_sep) ? 1u : 0u) | ((zero_area || s13_sep) ? 2u : 0u) |
             ((zero_area || s23_sep) ? 4u : 0u);
    }
  }
  // the winner is run once more on s itself (the same result) instead of
  // keeping a copy of its simplex
  float best = -1.f;
  int bk = -1;
#pragma unroll 1
  for (int k = 0; k < 3; ++k) {
    if (!(cand & (1u << k))) continue;
    Simplex c = s;
    if (k == 0) {
      c.copy(0, 1);
      c.copy(1, 2);
    } else if (k == 1) {
      c.copy(1, 2);
    }
    c.rank = 2;
    f3 pt;
    update2(c, pt, tol);
    const float dd = sqn(pt);
    if (best < 0.f || dd < best) { best = dd; bk = k; }
  }
  if (bk < 0) {
    out = n * (dot(s1, n) / area2);
    return;
  }
  if (bk == 0) {
    s.copy(0, 1);
    s.copy(1, 2);
  } else if (bk == 1) {
    s.copy(1, 2);
  }
  s.rank = 2;
  update2(s, out, tol);
}

// gjk_distance.hpp:288-373 (slot 3 newest): best of faces (3,2,1), (3,2,0),
// (3,1,0), through one update3 call site.
__device__ FCLG_GJK_COLD Upd update4(Simplex& s, f3& out, float tol) {
  // k = 0..2 the three faces, k = 3 the winner once more on s itself (the
  // same result; no copy of its simplex is kept)
  float best = -1.f;
  int bk = 0;
#pragma unroll 1
  for (int k = 0; k < 4; ++k) {
    const int f = k < 3 ? k : bk;
    Simplex c = s;
    if (f == 0) {
      c.copy(0, 1); c.copy(1, 2); c.copy(2, 3);
    } else if (f == 1) {
      c.copy(1, 2); c.copy(2, 3);
    } else {
      c.copy(2, 3);
    }
    c.rank = 3;
    f3 pt;
    update3(c, pt, tol);
    if (k == 3) {
      s = c;
      out = pt;
      break;
    }
    const float dd = sqn(pt);
    if (best < 0.f || dd < best) { best = dd; bk = k; }
  }
  return Upd::OK;
}

__device__ __forceinline__ Upd update_simplex(Simplex& s, f3& out, float tol) {
  if (s.rank == 1) { out = s.w[0]; return Upd::OK; }
  if (s.rank == 2) { update2(s, out, tol); return Upd::OK; }
  if (s.rank == 3) { update3(s, out, tol); return Upd::OK; }
  if (s.rank == 4) return update4(s, out, tol);
  return Upd::Failed;
}

// gjk_distance.hpp:375-470; the stored support points replace the
// reference's re-evaluation of support0/support1 at the stored directions.
__device__ FCLG_GJK_COLD bool extract_no_sub(const Simplex& s, f3& p0, f3& p1) {
  constexpr float kBaryTol = 1e-3f;
  if (s.rank == 4 || s.rank < 1) return false;
  if (s.rank == 1) {
    p0 = s.a[0];
    p1 = s.b[0];
    return true;
  }
  if (s.rank == 2) {
    const f3 s1_to_s2 = s.w[1] - s.w[0];
    const float len2 = sqn(s1_to_s2);
    if (len2 <= 0.f) {
      p0 = s.a[0];
      p1 = s.b[0];
      return true;
    }
    const float w2 = -dot(s.w[0], s1_to_s2) / len2;
    if (w2 > 1.f + kBaryTol) { p0 = s.a[1]; p1 = s.b[1]; return false; }
    if (w2 < -kBaryTol) { p0 = s.a[0]; p1 = s.b[0]; return false; }
    const float w1 = 1.f - w2;
    p0 = s.a[0] * w1 + s.a[1] * w2;
    p1 = s.b[0] * w1 + s.b[1] * w2;
    return true;
  }
  // Triangle.  FP32 when the triangle is well shaped (sin^2 of its angle at
  // vertex 0 >= 1e-4) and the origin projects inside it; otherwise the
  // barycentric solve reruns in FP64 on the FP32 support points: on a sliver
  // (near-collinear support points, common on curved surfaces) FP32 area
  // ratios lose every digit and the witness points can land centimetres
  // from the simplex's closest point.
  {
    const f3 s1_to_s2 = s.w[1] - s.w[0], s1_to_s3 = s.w[2] - s.w[0];
    const f3 n = cross(s1_to_s2, s1_to_s3);
    const float area2 = sqn(n);
    if (area2 > 1e-4f * sqn(s1_to_s2) * sqn(s1_to_s3)) {
      const f3 proj = n * (dot(s.w[0], n) / area2);
      const float area = sqrtf(area2);
      const float w2 = nrm(cross(s1_to_s3, s.w[0] - proj)) / area;
      const float w3 = nrm(cross(s1_to_s2, s.w[0] - proj)) / area;
      const float w1 = 1.f - w2 - w3;
      if (w1 >= -kBaryTol && w2 >= -kBaryTol && w3 >= -kBaryTol) {
        p0 = (s.a[0] * w1 + s.a[1] * w2) + s.a[2] * w3;
        p1 = (s.b[0] * w1 + s.b[1] * w2) + s.b[2] * w3;
        return true;
      }
    }
  }
  const auto tof = [](d3 v) { return mk3((float)v.x, (float)v.y, (float)v.z); };
  const d3 a0 = tod(s.a[0]), a1 = tod(s.a[1]), a2 = tod(s.a[2]);
  const d3 b0 = tod(s.b[0]), b1 = tod(s.b[1]), b2 = tod(s.b[2]);
  const d3 w0 = a0 - b0, w1v = a1 - b1, w2v = a2 - b2;
  const d3 s1_to_s2 = w1v - w0, s1_to_s3 = w2v - w0;
  const d3 n = cross(s1_to_s2, s1_to_s3);
  const double area2 = dot(n, n);
  if (area2 <= 0.0) return false;
  const d3 proj = n * (dot(w0, n) / area2);
  const double area = sqrt(area2);
  const d3 c2 = cross(s1_to_s3, w0 - proj), c3 = cross(s1_to_s2, w0 - proj);
  double u2 = sqrt(dot(c2, c2)) / area;
  double u3 = sqrt(dot(c3, c3)) / area;
  double u1 = 1.0 - u2 - u3;
  if (u1 < -(double)kBaryTol || u2 < -(double)kBaryTol || u3 < -(double)kBaryTol) {
    // The FP32 iterates converged on this triangle, but its exact closest
    // point lies on an edge or vertex (a sliver's weights move by more than
    // the tolerance under FP32 rounding of the support points): take that
    // point, where the reference would report no witness.
    closest_bary_origin(w0, w1v, w2v, u1, u2, u3);
  }
  p0 = tof((a0 * u1 + a1 * u2) + a2 * u3);
  p1 = tof((b0 * u1 + b1 * u2) + b2 * u3);
  return true;
}

// gjk_distance.hpp:472-559
__device__ FCLG_GJK_COLD bool extract_try_sub(const Simplex& s, f3& p0, f3& p1) {
  if (s.rank >= 4) return false;
  if (s.rank <= 2) {
    extract_no_sub(s, p0, p1);
    return true;
  }
  float best = -1.f;
  f3 b0 = mk3(0, 0, 0), b1 = mk3(0, 0, 0), c0, c1;
  Simplex c = s;
  if (extract_no_sub(c, c0, c1)) {
    const float dd = sqn(c0 - c1);
    if (best < 0.f || dd < best) { best = dd; b0 = c0; b1 = c1; }
  }
  c = s;
  c.rank = 2;
  extract_no_sub(c, c0, c1);
  float dd = sqn(c0 - c1);
  if (best < 0.f || dd < best) { best = dd; b0 = c0; b1 = c1; }
  c = s;
  c.copy(1, 2);
  c.rank = 2;
  extract_no_sub(c, c0, c1);
  dd = sqn(c0 - c1);
  if (best < 0.f || dd < best) { best = dd; b0 = c0; b1 = c1; }
  c = s;
  c.copy(0, 1);
  c.copy(1, 2);
  c.rank = 2;
  extract_no_sub(c, c0, c1);
  dd = sqn(c0 - c1);
  if (best < 0.f || dd < best) { best = dd; b0 = c0; b1 = c1; }
  p0 = b0;
  p1 = b1;
  return true;
}

// GJK boolean (gjk.hpp:10-140) then, for a separating vertex, the minimum
// distance loop (gjk_distance.hpp:10-105) as a machine that advances by one
// support evaluation per step(): begin() sets it up, step() returns true once
// o holds the answer.  The refilling GJK pass (gjk_pass.cuh) interleaves the
// steps of 32 pairs per warp and hands a finished lane its next pair.  The
// same decisions in the same order as gjk_evaluate / min_distance below (the
// loop form, which the group-per-pair pass keeps: its register allocation
// does not survive the machine form); the two passes' answers are compared
// bit for bit in the tests.
struct GjkRun {
  Simplex s;
  f3 d;        // boolean: search direction; distance: next direction
  f3 cur;      // distance: current closest point of the simplex
  float book;  // distance: |cur|
  int phase;   // 0 first support, 1 boolean loop, 2 distance loop, 3 done
  int it;      // iteration of the current loop
  int probe;   // > 0: supports the boolean phase may take (gjk_evaluate's probe)
  float cert;  // > 0: certified distance stop (min_distance's cert_gap)
  GjkOut o;

  __device__ __forceinline__ void begin(f3 guess, int probe_supports = 0, float cert_gap = 0.f) {
    probe = probe_supports;
    cert = cert_gap;
    o.point_valid = false;
    o.iterations = 0;
    o.p0 = o.p1 = mk3(0, 0, 0);
    d = guess;
    if (sqn(d) <= 0.f) d = mk3(1, 0, 0);
    d = normalized(d);
    phase = 0;
    it = 0;
  }

  __device__ __forceinline__ bool done() {
    phase = 3;
    return true;
  }

  // gjk.hpp:112-140 for the undetermined outcomes (no progress, iteration limit)
  __device__ __forceinline__ bool undetermined(int status, bool want_distance) {
    o.status = status;
    if (want_distance) o.point_valid = extract_try_sub(s, o.p0, o.p1);
    return done();
  }

  __device__ __forceinline__ bool distance_result(bool valid) {
    o.point_valid = valid && extract_no_sub(s, o.p0, o.p1);
    return done();
  }

  // separated: the rank-1 simplex s seeds the distance loop (gjk_distance.hpp:10-40)
  __device__ __forceinline__ bool enter_distance(float tol, int max_iter, bool want_distance) {
    o.status = kGjkSeparated;
    s.rank = 1;
    if (!want_distance) return done();
    if (update_simplex(s, cur, tol) != Upd::OK) return done();
    book = nrm(cur);
    if (book <= tol) return distance_result(true);
    d = cur * (-1.f / book);
    phase = 2;
    it = 0;
    if (max_iter <= 0) return done();
    return false;
  }

  // boolean iterations allowed: max_iter, or fewer under a probe
  __device__ __forceinline__ int bool_iters(int max_iter) const {
    return (probe > 0 && probe - 1 < max_iter) ? probe - 1 : max_iter;
  }
  __device__ __forceinline__ bool boolean_limit(int max_iter, bool want_distance) {
    if (bool_iters(max_iter) < max_iter) {  // the learned start's probe ran out
      o.status = kGjkIterLimit;
      return done();
    }
    return undetermined(kGjkIterLimit, want_distance);
  }

  template <class Sup>
  __device__ __forceinline__ bool step(const Sup& sup, float tol, int max_iter, bool want_distance) {
    const float tol2 = tol * tol;
    // every phase supports along d: one call site, so that lanes of a warp in
    // different phases still evaluate their supports together
    f3 pa, pb;
    sup(d, pa, pb);
    if (phase == 0) {
      s.set(0, pa, pb);
      s.rank = 1;
      if (sqn(s.w[0]) <= tol2) {
        o.status = kGjkIntersect;
        return done();
      }
      if (dot(s.w[0], d) < 0.f) return enter_distance(tol, max_iter, want_distance);
      d = -d;
      phase = 1;
      it = 0;
      if (bool_iters(max_iter) <= 0) return boolean_limit(max_iter, want_distance);
      return false;
    }
    if (phase == 1) {
      o.iterations = it + 1;
      const f3 w = pa - pb;
      if (dot(w, d) < 0.f) {
        s.set(0, pa, pb);  // the separating vertex seeds the distance simplex
        return enter_distance(tol, max_iter, want_distance);
      }
      bool dup = false;
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (j < s.rank && sqn(s.w[j] - w) < tol2) dup = true;
      if (dup) return undetermined(kGjkNoProgress, want_distance);
      if (s.rank == 1) s.set(1, pa, pb);
      else if (s.rank == 2) s.set(2, pa, pb);
      else s.set(3, pa, pb);
      s.rank += 1;
      if (sqn(w) <= tol2) {
        o.status = kGjkIntersect;
        return done();
      }
      Proj st;
      if (s.rank == 2) st = project2(s, d);
      else if (s.rank == 3) st = project3(s, d, tol);
      else st = project4(s, d, tol);
      if (st == Proj::Failed) {
        o.status = kGjkFailed;
        return done();
      }
      if (st == Proj::Intersect) {
        o.status = kGjkIntersect;
        return done();
      }
      if (st == Proj::ZeroVolume) return undetermined(kGjkNoProgress, want_distance);
      if (++it >= bool_iters(max_iter)) return boolean_limit(max_iter, want_distance);
      return false;
    }
    // phase 2: one iteration of the minimum-distance loop (gjk_distance.hpp:41-105)
    ++o.iterations;
    const f3 w = pa - pb;
    const float gap = dot(d, w - cur);
    FCLG_GJK_TRACE(it, -1, gap, 0.f);
    if (gap < tol) return distance_result(true);
    bool dup = false;
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (j < s.rank && sqn(s.w[j] - w) < tol2) dup = true;
    if (dup) return distance_result(true);
    // s.rank is 1..3 here
    if (s.rank == 1) s.set(1, pa, pb);
    else if (s.rank == 2) s.set(2, pa, pb);
    else s.set(3, pa, pb);
    s.rank += 1;
    const Upd st = update_simplex(s, cur, tol);
    if (st == Upd::NoImprovement) return distance_result(true);
    if (st != Upd::OK) return done();
    const float nd = nrm(cur);
    FCLG_GJK_TRACE(it, s.rank, nd, book - nd);
    if (book - nd < tol) {
      if (!(cert > 0.f) || gap <= cert) return distance_result(true);
      if (!(book - nd > 0.f)) return done();  // no progress before the certificate: point_valid stays false
    }
    if (nd < tol) return distance_result(true);
    book = nd;
    d = cur * (-1.f / book);
    if (++it >= max_iter) return done();
    return false;
  }
};

// gjk_distance.hpp:10-105: minimum distance from a separating vertex.
// cert_gap > 0 (runs from a learned start) replaces the reference's stop on a
// small improvement with a certificate: the run ends on a small improvement
// only once the duality gap of the last support, |v| - v^.w (an upper bound of
// |v| - distance), is at most cert_gap, and gives up (returns false, so the
// pair is redone from the plain start) when an iteration makes no progress
// before that.
template <class Sup>
__device__ __forceinline__ bool min_distance(const Sup& sup, Simplex& s, float tol, int max_iter, f3& p0, f3& p1,
                                             int& iters, float cert_gap = 0.f) {
  // every stop that extracts the witness points leaves the loop to the one
  // extract_no_sub call at the end (one copy of its code)
  if (s.rank != 1) return false;
  f3 cur = s.w[0];
  float book = nrm(cur);
  bool extract = book <= tol;
  if (!extract) {
    f3 next = cur * (-1.f / book);
    const float tol2 = tol * tol;
    for (int it = 0; it < max_iter; ++it) {
      ++iters;
      f3 pa, pb;
      sup(next, pa, pb);
      const f3 w = pa - pb;
      const float gap = dot(next, w - cur);
      FCLG_GJK_TRACE(it, -1, gap, 0.f);
      if (gap < tol) { extract = true; break; }
      bool dup = false;
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (j < s.rank && sqn(s.w[j] - w) < tol2) dup = true;
      if (dup) { extract = true; break; }
      // s.rank is 1..3 here
      if (s.rank == 1) s.set(1, pa, pb);
      else if (s.rank == 2) s.set(2, pa, pb);
      else s.set(3, pa, pb);
      s.rank += 1;
      const Upd st = update_simplex(s, cur, tol);
      if (st == Upd::NoImprovement) { extract = true; break; }
      if (st != Upd::OK) break;
      const float nd = nrm(cur);
      FCLG_GJK_TRACE(it, s.rank, nd, book - nd);
      if (book - nd < tol) {
        if (!(cert_gap > 0.f) || gap <= cert_gap) { extract = true; break; }
        if (!(book - nd > 0.f)) break;
      }
      if (nd < tol) { extract = true; break; }
      book = nd;
      next = cur * (-1.f / book);
    }
  }
  return extract && extract_no_sub(s, p0, p1);
}

// Outcome of the boolean phase (gjk_boolean): the run is over (o.status set),
// separation is certified (s holds the separating vertex as a rank-1 simplex:
// the distance loop starts there), or the loop stopped undetermined (o.status
// set; the witness points come from the simplex by extract_try_sub).
enum : int { kBoolDone = 0, kBoolSeparated = 1, kBoolUndetermined = 2 };

// The boolean phase of gjk.hpp:10-140.  probe > 0 (a learned start) allows it
// that many support evaluations to certify separation; past them the run ends
// with kGjkIterLimit and no points (the pair is then redone from the plain
// start).  o.iterations counts its loop iterations.
template <class Sup>
__device__ __forceinline__ int gjk_boolean(const Sup& sup, f3 guess, float tol, int max_iter, Simplex& s, GjkOut& o,
                                           int probe = 0) {
  f3 d = guess;
  if (sqn(d) <= 0.f) d = mk3(1, 0, 0);
  d = normalized(d);
  const float tol2 = tol * tol;
  f3 pa, pb;
  sup(d, pa, pb);
  s.set(0, pa, pb);
  s.rank = 1;
  if (sqn(s.w[0]) <= tol2) { o.status = kGjkIntersect; return kBoolDone; }
  if (dot(s.w[0], d) < 0.f) return kBoolSeparated;
  d = -d;
  const int bool_iters = (probe > 0 && probe - 1 < max_iter) ? probe - 1 : max_iter;
  for (int it = 0; it < bool_iters; ++it) {
    o.iterations = it + 1;
    sup(d, pa, pb);
    const f3 w = pa - pb;
    if (dot(w, d) < 0.f) {
      s.set(0, pa, pb);  // the separating vertex seeds the distance simplex
      s.rank = 1;
      return kBoolSeparated;
    }
    bool dup = false;
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (j < s.rank && sqn(s.w[j] - w) < tol2) dup = true;
    if (dup) { o.status = kGjkNoProgress; return kBoolUndetermined; }
    if (s.rank == 1) s.set(1, pa, pb);
    else if (s.rank == 2) s.set(2, pa, pb);
    else s.set(3, pa, pb);
    s.rank += 1;
    if (sqn(w) <= tol2) { o.status = kGjkIntersect; return kBoolDone; }
    Proj st;
    if (s.rank == 2) st = project2(s, d);
    else if (s.rank == 3) st = project3(s, d, tol);
    else st = project4(s, d, tol);
    if (st == Proj::Failed) { o.status = kGjkFailed; return kBoolDone; }
    if (st == Proj::Intersect) { o.status = kGjkIntersect; return kBoolDone; }
    if (st == Proj::ZeroVolume) { o.status = kGjkNoProgress; return kBoolUndetermined; }
  }
  o.status = kGjkIterLimit;
  // the learned start's probe ran out: no points
  return bool_iters < max_iter ? kBoolDone : kBoolUndetermined;
}

// gjk.hpp:10-140.  want_distance selects the MinSeparationDistanceOutput path.
// probe: see gjk_boolean; cert_gap: see min_distance.
template <class Sup>
__device__ __forceinline__ GjkOut gjk_evaluate(const Sup& sup, f3 guess, float tol, int max_iter, bool want_distance,
                                               Simplex& s, int probe = 0, float cert_gap = 0.f) {
  GjkOut o;
  o.point_valid = false;
  o.iterations = 0;
  o.p0 = o.p1 = mk3(0, 0, 0);
  const int k = gjk_boolean(sup, guess, tol, max_iter, s, o, probe);
  if (k == kBoolSeparated) {
    o.status = kGjkSeparated;
    if (want_distance) o.point_valid = min_distance(sup, s, tol, max_iter, o.p0, o.p1, o.iterations, cert_gap);
  } else if (k == kBoolUndetermined && want_distance) {
    o.point_valid = extract_try_sub(s, o.p0, o.p1);
  }
  return o;
}

}  // namespace fclg
