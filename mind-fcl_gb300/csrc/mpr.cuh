// MPR boolean intersection (Minkowski portal refinement), the test
// fcl::collide runs for a shape pair when no contact is requested
// (ShapeIntersectIndepImpl::run, gjk_solver-inl.h:70-137, which falls back to
// GJK when MPR reports failure).  Restates MPR::RunIntersect and its helpers
// (cvx_collide/mpr.hpp:10-15, 33-185, 187-328, 434-493) in FP32, one thread
// (or lane group) per pair.
#pragma once
#include "support.cuh"

namespace fclg {

enum class MprStatus : int { Intersect = 0, Separated = 1, Failed = 2 };

// MPR::IntersectData (mpr.h:23-31) at an Intersect exit: the interior point,
// the portal and the (unit) directions that found its vertices; `count` of
// v1..v3 set (0: the interior point is at the origin; 1: the origin lies on
// the segment v0 v1; 3: inside the tetrahedron v0 v1 v2 v3).
struct MprPortal {
  f3 v0, v1, v2, v3, d1, d2, d3;
  int count;
};

// Interior point of a shape in its own frame: the vertex mean of a hull
// (convex-inl.h:58-63, stored in fclg_shape.param[0:3]), the origin otherwise.
__device__ __forceinline__ f3 load_interior(const int4* __restrict__ shapes, uint32_t i, int type) {
  if (type != kConvex && type != kConvexWalk) return mk3(0.f, 0.f, 0.f);
  const float4 p = __ldg(reinterpret_cast<const float4*>(shapes) + 2 * (size_t)i + 1);
  return mk3(p.x, p.y, p.z);
}

// mpr.hpp:18-20: the tolerance tests use the L1 norm.
__device__ __forceinline__ float absnorm(f3 v) { return fabsf(v.x) + fabsf(v.y) + fabsf(v.z); }

template <class Sup>
struct Mpr {
  const Sup& sup;
  int max_iter;
  float tol;
  int iterations = 0;

  // mpr.hpp:10-15: the direction is normalised in place, then supported.
  __device__ __forceinline__ f3 support(f3& d) const {
    d = normalized(d);
    f3 pa, pb;
    sup(d, pa, pb);
    return pa - pb;
  }

  // mpr.hpp:187-328: 0 iteration limit, 1 separated, 2 portal found.
  __device__ int find_portal(f3 v0, f3& v1, f3& v2, f3& v3, f3& d1, f3& d2, f3& d3) {
    constexpr float kEps = 1.1920929e-07f;  // dot_eps_ratio = epsilon<T>() (mpr.h:103), T = float
    const float v0n = absnorm(v0);
    for (int it = 0;; ++it) {
      if (it >= max_iter) return 0;
      ++iterations;
      f3 a1 = v1 - v0, a2 = v2 - v0, a3 = v3 - v0;
      f3 n031 = cross(a3, a1);
      f3 n012 = cross(a1, a2);
      if (dot(a2, n031) < 0.f) {
        f3 t = v2; v2 = v3; v3 = t;
        t = d2; d2 = d3; d3 = t;
        t = a2; a2 = a3; a3 = t;
        t = n012; n012 = n031; n031 = t;
        n031 = -n031;
        n012 = -n012;
      }
      if (dot(v0, n031) > kEps * v0n * absnorm(n031)) {
        f3 sd = -n031;
        v2 = support(sd);
        d2 = sd;
        if (dot(v2, sd) < 0.f) return 1;
        continue;
      }
      if (dot(v0, n012) > kEps * v0n * absnorm(n012)) {
        f3 sd = -n012;
        v3 = support(sd);
        d3 = sd;
        if (dot(v3, sd) < 0.f) return 1;
        continue;
      }
      const f3 n023 = cross(a2, a3);
      if (dot(v0, n023) > kEps * v0n * absnorm(n023)) {
        f3 sd = -n023;
        v1 = support(sd);
        d1 = sd;
        if (dot(v1, sd) < 0.f) return 1;
        continue;
      }
      return 2;
    }
  }

  // mpr.hpp:434-493
  __device__ __forceinline__ static void update_portal(f3 v0, f3 v4, f3 n, f3& v1, f3& v2, f3& v3, f3& d1, f3& d2,
                                                       f3& d3) {
    const f3 pn = cross(v4, v0);
    if (dot(v1, pn) > 0.f) {
      if (dot(v2, pn) > 0.f) { v1 = v4; d1 = n; }
      else { v3 = v4; d3 = n; }
    } else {
      if (dot(v3, pn) > 0.f) { v2 = v4; d2 = n; }
      else { v1 = v4; d1 = n; }
    }
  }

  // Directed penetration, mpr.hpp:495-595 and :606-701: the depth of the
  // Minkowski difference along the unit direction d (shape b's escape
  // direction in a's frame) and witness points p0 / p1.  Returns 0 OK,
  // 1 Failed, 2 FailedNoIntersect, 3 FailedRefinementIterationLimit.
  __device__ int directed(f3 d, float& depth, f3& p0, f3& p1) {
    iterations = 0;
    const f3 v0 = -d;
    f3 d1 = d;
    f3 v1 = support(d1);
    if (dot(d1, v1) < 0.f) return 2;
    f3 d2 = cross(v0, v1);
    if (absnorm(d2) <= absnorm(v1) * tol) {
      depth = dot(v1, d);
      sup(d1, p0, p1);
      return 0;
    }
    f3 v2 = support(d2);
    if (dot(d2, v2) < 0.f) return 2;
    f3 d3 = cross(v1, v2);
    if (dot(d3, v0) > 0.f) {
      f3 t = v1; v1 = v2; v2 = t;
      t = d1; d1 = d2; d2 = t;
      d3 = -d3;
    }
    f3 v3 = support(d3);
    if (dot(d3, v3) < 0.f) return 2;
    const float m2 = fmaxf(sqn(v1), fmaxf(sqn(v2), sqn(v3)));
    const f3 v0s = v0 * sqrtf(m2);
    const int fp = find_portal(v0s, v1, v2, v3, d1, d2, d3);
    if (fp == 0) return 1;
    if (fp == 1) return 2;
    for (int it = 0; it < max_iter; ++it) {
      ++iterations;
      f3 n = cross(v2 - v1, v3 - v1);
      if (dot(n, d) < 0.f) {
        f3 t = v2; v2 = v3; v3 = t;
        t = d2; d2 = d3; d3 = t;
        n = -n;
      }
      const f3 v4 = support(n);
      if (dot(v4, n) < 0.f) return 2;
      if (fabsf(dot(v4 - v1, n)) < tol * absnorm(n)) {
        // finalizeDirectedPenetrationResult (mpr.hpp:606-701) with v4
        const float ndd = dot(d, n);
        if (!(fabsf(ndd) > 0.f)) {
          const float a1 = dot(v1, d), a2 = dot(v2, d), a3 = dot(v3, d);
          f3 db = d1;
          depth = a1;
          if (a2 > depth) { depth = a2; db = d2; }
          if (a3 > depth) { depth = a3; db = d3; }
          sup(db, p0, p1);
          return 0;
        }
        const float dist_v123 = dot(v1, n) / ndd;
        depth = dot(v4, n) / ndd;
        const f3 o_proj = d * dist_v123;
        const f3 a12 = v2 - v1, a13 = v3 - v1;
        const float area = nrm(cross(a12, a13));
        const float w2 = nrm(cross(a13, v1 - o_proj)) / area;
        const float w3 = nrm(cross(a12, v1 - o_proj)) / area;
        const float w1 = 1.f - w2 - w3;
        f3 pa1, pb1, pa2, pb2, pa3, pb3;
        sup(d1, pa1, pb1);
        sup(d2, pa2, pb2);
        sup(d3, pa3, pb3);
        p0 = (pa1 * w1 + pa2 * w2) + pa3 * w3;
        p1 = (pb1 * w1 + pb2 * w2) + pb3 * w3;
        return 0;
      }
      update_portal(v0s, v4, n, v1, v2, v3, d1, d2, d3);
    }
    return 3;
  }

  // mpr.hpp:33-185.  v0 is the interior point of the Minkowski difference.
  // Incremental minimum-distance penetration from the unit hint d
  // (mpr_incremental_penetration.hpp:176-288, return on the first converged
  // subroutine, as fcl::collide calls it): explore d -- the MPR portal along
  // d, refined until its supporting plane either converges (done) or bounds
  // the depth along d below the depth along the portal normal (continue
  // along that normal).  0 OK, 1 Failed, 2 FailedNoIntersect, 4 iteration
  // limit (still a valid penetration); depth, direction and witness points.
  __device__ int incremental(f3 d, float& depth, f3& dir, f3& p0, f3& p1) {
    iterations = 0;
    f3 v1 = mk3(0, 0, 0), v2 = v1, v3 = v1, d1 = v1, d2 = v1, d3 = v1;
    float prev_lb = -1.f, prev_ub = -1.f;
    for (int outer = 0; outer < max_iter; ++outer) {
      f3 nd = d;
      float lb = 0.f, ub = 0.f;
      const int st = explore(d, v1, v2, v3, d1, d2, d3, lb, ub, nd, outer >= 1);
      if (st == 0) {
        d = nd;
      } else if (st == 1) {
        finish_incremental(d, v1, v2, v3, d1, d2, d3, lb, ub, depth, dir, p0, p1);
        return 0;
      } else if (st == 2) {
        depth = ub;
        dir = nd;
        sup(nd, p0, p1);
        return 0;
      } else {
        return st == 4 ? 2 : 1;
      }
      prev_lb = lb;
      prev_ub = ub;
    }
    finish_incremental(d, v1, v2, v3, d1, d2, d3, prev_lb, prev_ub, depth, dir, p0, p1);
    return 4;
  }

  // mpr_incremental_penetration.hpp:49-174: 0 new direction, 1 converged,
  // 2 degenerated, 3 failed, 4 no intersection.  lb / ub bound the depth
  // along d (:10-47).
  __device__ int explore(f3 d, f3& v1, f3& v2, f3& v3, f3& d1, f3& d2, f3& d3, float& lb, float& ub, f3& nd,
                         bool v123_valid) {
    const f3 v0 = -d;
    f3 init_dir = d;
    const f3 init = support(init_dir);
    if (dot(d, init) < 0.f) return 4;
    if (!v123_valid) {
      d1 = d;
      v1 = init;
      d2 = cross(v0, v1);
      if (absnorm(d2) <= absnorm(v1) * tol) {
        lb = dot(v1, d);
        ub = lb;
        nd = d;
        return 2;
      }
      v2 = support(d2);
      if (dot(d2, v2) < 0.f) return 4;
      d3 = cross(v1, v2);
      if (dot(d3, v0) > 0.f) {
        f3 t = v1; v1 = v2; v2 = t;
        t = d1; d1 = d2; d2 = t;
        d3 = -d3;
      }
      v3 = support(d3);
      if (dot(d3, v3) < 0.f) return 4;
    }
    const float m2 = fmaxf(sqn(v1), fmaxf(sqn(v2), sqn(v3)));
    const f3 v0s = v0 * sqrtf(m2);
    const int fp = find_portal(v0s, v1, v2, v3, d1, d2, d3);
    if (fp == 0) return 3;
    if (fp == 1) return 4;
    for (int it = 0; it < max_iter; ++it) {
      ++iterations;
      f3 n = cross(v2 - v1, v3 - v1);
      if (dot(n, d) < 0.f) {
        f3 t = v2; v2 = v3; v3 = t;
        t = d2; d2 = d3; d3 = t;
        n = -n;
      }
      const f3 v4 = support(n);
      const float ub_plane = dot(v4, n);
      if (ub_plane < 0.f) return 4;
      const float v1n = dot(v1, n), v4n = dot(v4, n);
      const float ndd = dot(d, n);
      if (fabsf(ndd) <= 0.f) {  // as the reference tests it (a NaN takes the division)
        lb = fmaxf(dot(v1, d), fmaxf(dot(v2, d), dot(v3, d)));
        ub = lb;
      } else {
        lb = v1n / ndd;
        ub = v4n / ndd;
      }
      if (lb > ub_plane + tol) {
        nd = n;
        return 0;
      }
      if (fabsf(v4n - v1n) <= tol) {
        nd = n;
        return 1;
      }
      update_portal(v0s, v4, n, v1, v2, v3, d1, d2, d3);
    }
    return 3;
  }

  // finalizeIncrementalPenetrationResult (mpr_incremental_penetration.hpp:300-333)
  __device__ void finish_incremental(f3 d, f3 v1, f3 v2, f3 v3, f3 d1, f3 d2, f3 d3, float lb, float ub,
                                     float& depth, f3& dir, f3& p0, f3& p1) const {
    depth = ub;
    dir = d;
    const f3 o_proj = d * lb;
    const f3 a12 = v2 - v1, a13 = v3 - v1;
    const float area = nrm(cross(a12, a13));
    const float w2 = nrm(cross(a13, v1 - o_proj)) / area;
    const float w3 = nrm(cross(a12, v1 - o_proj)) / area;
    const float w1 = 1.f - w2 - w3;
    f3 pa1, pb1, pa2, pb2, pa3, pb3;
    sup(d1, pa1, pb1);
    sup(d2, pa2, pb2);
    sup(d3, pa3, pb3);
    p0 = (pa1 * w1 + pa2 * w2) + pa3 * w3;
    p1 = (pb1 * w1 + pb2 * w2) + pb3 * w3;
  }

  // KEEP: the portal of an Intersect exit is written to *keep.
  template <bool KEEP = false>
  __device__ MprStatus intersect(f3 v0, MprPortal* keep = nullptr) {
    iterations = 0;
    if (sqn(v0) <= tol * tol) {
      if constexpr (KEEP) keep->v0 = v0, keep->count = 0;
      return MprStatus::Intersect;
    }
    f3 d1 = -v0;
    f3 v1 = support(d1);
    if (dot(d1, v1) < 0.f) return MprStatus::Separated;
    f3 d2 = cross(v0, v1);
    if (absnorm(d2) <= absnorm(v0) * absnorm(v1) * tol) {
      if constexpr (KEEP) keep->v0 = v0, keep->v1 = v1, keep->d1 = d1, keep->count = 1;
      return MprStatus::Intersect;
    }
    f3 v2 = support(d2);
    if (dot(d2, v2) < 0.f) return MprStatus::Separated;
    f3 d3 = cross(v1 - v0, v2 - v0);
    if (dot(d3, v0) > 0.f) {
      f3 t = v1; v1 = v2; v2 = t;
      t = d1; d1 = d2; d2 = t;
      d3 = -d3;
    }
    f3 v3 = support(d3);
    if (dot(d3, v3) < 0.f) return MprStatus::Separated;
    const int fp = find_portal(v0, v1, v2, v3, d1, d2, d3);
    if (fp == 0) return MprStatus::Failed;
    if (fp == 1) return MprStatus::Separated;
    for (int it = 0; it < max_iter; ++it) {
      ++iterations;
      f3 n = cross(v2 - v1, v3 - v1);
      if (dot(n, v0) > 0.f) {
        f3 t = v2; v2 = v3; v3 = t;
        t = d2; d2 = d3; d3 = t;
        n = -n;
      }
      if (!(dot(v1, n) < 0.f)) {
        if constexpr (KEEP) *keep = MprPortal{v0, v1, v2, v3, d1, d2, d3, 3};
        return MprStatus::Intersect;
      }
      const f3 v4 = support(n);
      if (dot(v4, n) < 0.f) return MprStatus::Separated;
      if (fabsf(dot(v4 - v1, n)) < tol * absnorm(n)) return MprStatus::Separated;
      update_portal(v0, v4, n, v1, v2, v3, d1, d2, d3);
    }
    return MprStatus::Failed;
  }
};

}  // namespace fclg
