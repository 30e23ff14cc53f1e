// Support mappings of the five shape types and of their Minkowski difference,
// evaluated cooperatively by a group of LANES lanes (LANES = 1: one thread per
// pair; 32: one warp per pair).
//
// Primitive supports restate gjk_shape.hpp:44-51 (box), :65-71 (sphere),
// :101-117 (capsule), :161-177 (cylinder) in FP32.  The convex support is the
// argmax of d.v over the hull's vertices (convex-inl.h:133-149): every lane of
// the group scans a strided slice of the vertex list with vectorised float4
// loads, then a shuffle butterfly reduces (value, index) pairs, lowest index
// winning ties as the reference's first-maximum scan does.
#pragma once
#include "device_math.cuh"

namespace fclg {

template <int LANES>
struct Group {
  unsigned lane;   // lane within the group
  unsigned mask;   // member mask of the group within the warp
  unsigned base;   // warp lane of the group's first lane
  __device__ __forceinline__ static Group make() {
    Group g;
    const unsigned wl = threadIdx.x & 31u;
    g.lane = wl & (LANES - 1);
    g.base = wl & ~(unsigned)(LANES - 1);
    g.mask = (LANES == 32) ? 0xFFFFFFFFu : (((1u << LANES) - 1u) << g.base);
    return g;
  }
};

template <int LANES>
__device__ __forceinline__ f3 convex_support(const float4* __restrict__ v, uint32_t nv, f3 d, const Group<LANES>& g) {
  float best;
  uint32_t bi;
  if (g.lane == 0 && nv > 0) {
    const float4 q = __ldg(v);
    best = fmaf(d.z, q.z, fmaf(d.y, q.y, d.x * q.x));
    bi = 0;
  } else {
    best = -INFINITY;
    bi = 0xFFFFFFFFu;
  }
  uint32_t i = (g.lane == 0) ? LANES : g.lane;
#pragma unroll 4
  for (; i < nv; i += LANES) {
    const float4 q = __ldg(v + i);
    const float val = fmaf(d.z, q.z, fmaf(d.y, q.y, d.x * q.x));
    if (val > best) {
      best = val;
      bi = i;
    }
  }
  if constexpr (LANES == 32) {
    // warp argmax by two reductions: the largest value (an order-preserving
    // map to unsigned; -0 taken as +0, NaN below everything), then the
    // lowest index holding it
    best += 0.f;
    const uint32_t vb = __float_as_uint(best);
    const uint32_t u = (best != best) ? 0u : ((vb & 0x80000000u) ? ~vb : (vb | 0x80000000u));
    const uint32_t umax = __reduce_max_sync(0xFFFFFFFFu, u);
    bi = __reduce_min_sync(0xFFFFFFFFu, u == umax ? bi : 0xFFFFFFFFu);
  } else if (LANES > 1) {
#pragma unroll
    for (int off = LANES / 2; off > 0; off >>= 1) {
      const float ov = __shfl_xor_sync(g.mask, best, off);
      const uint32_t oi = __shfl_xor_sync(g.mask, bi, off);
      if (ov > best || (ov == best && oi < bi)) {
        best = ov;
        bi = oi;
      }
    }
    // every lane must agree, also when a NaN direction made the order partial
    bi = __shfl_sync(g.mask, bi, g.base);
  }
  if (bi >= nv) bi = 0;
  const float4 q = __ldg(v + bi);
  return mk3(q.x, q.y, q.z);
}

// Hill climb over a walk block e (entries {x, y, z, link}, link = (row << 8) |
// degree).  Start: the cached corner of the axis direction with the largest
// d-component, the first of +x, -x, +y, -y, +z, -z on ties
// (convex-inl.h:206-222).  Step: scan the current corner's row, skipping the
// last two corners left behind; every strictly larger value moves the corner
// (convex-inl.h:230-278).  Values strictly increase, so no corner repeats; the
// pass count is bounded by the vertex count all the same.
__device__ __forceinline__ f3 convex_walk(const float4* __restrict__ e, uint32_t nv, f3 d) {
  int k = 0;
  float m = d.x;
  if (-d.x > m) { k = 1; m = -d.x; }
  if (d.y > m) { k = 2; m = d.y; }
  if (-d.y > m) { k = 3; m = -d.y; }
  if (d.z > m) { k = 4; m = d.z; }
  if (-d.z > m) k = 5;
  float4 cur = __ldg(e + k);
  float best = fmaf(d.z, cur.z, fmaf(d.y, cur.y, d.x * cur.x));
  uint32_t link = __float_as_uint(cur.w);
  uint32_t parent0 = link, parent1 = link;
  for (uint32_t pass = 0; pass < nv; ++pass) {
    const uint32_t row = link >> 8, deg = link & 0xFFu, from = link;
    for (uint32_t j = 0; j < deg; ++j) {
      const float4 q = __ldg(e + row + j);
      const uint32_t ql = __float_as_uint(q.w);
      if (ql == parent0 || ql == parent1) continue;
      const float v = fmaf(d.z, q.z, fmaf(d.y, q.y, d.x * q.x));
      if (v > best) {
        parent1 = link;
        link = ql;
        best = v;
        cur = q;
      }
    }
    parent0 = from;
    if (link == from) break;
  }
  return mk3(cur.x, cur.y, cur.z);
}

// pool: the vertex pool, or for kConvexWalk the walk blocks.
template <int LANES>
__device__ __forceinline__ f3 shape_support(const ShapeDev& s, const float4* __restrict__ pool, f3 d,
                                            const Group<LANES>& g) {
  switch (s.type) {
    case kBox:
      return mk3(d.x > 0.f ? s.p0 : -s.p0, d.y > 0.f ? s.p1 : -s.p1, d.z > 0.f ? s.p2 : -s.p2);
    case kSphere:
      return d * s.p0;
    case kCapsule: {
      const f3 v = d * s.p0;
      const f3 pos1 = mk3(v.x, v.y, s.p1 + v.z);
      const f3 pos2 = mk3(v.x, v.y, -s.p1 + v.z);
      return (dot(d, pos1) > dot(d, pos2)) ? pos1 : pos2;
    }
    case kCylinder: {
      const float zdist = sqrtf(fmaf(d.y, d.y, d.x * d.x));
      const float z = d.z > 0.f ? s.p1 : -s.p1;
      if (zdist == 0.f) return mk3(0.f, 0.f, z);
      const float k = s.p0 / zdist;
      return mk3(k * d.x, k * d.y, z);
    }
    case kConvex:
      return convex_support<LANES>(pool + s.vofs, s.nv, d, g);
    case kConvexWalk:
      if constexpr (LANES == 1) return convex_walk(pool + s.vofs, s.nv, d);
      return mk3(0.f, 0.f, 0.f);
    case kTriangle: {
      // triangleSupport, geometry/shape/shape_gjk_interface-inl.h:17-39
      const float4 qa = __ldg(pool + s.vofs), qb = __ldg(pool + s.vofs + 1), qc = __ldg(pool + s.vofs + 2);
      const f3 a = mk3(qa.x, qa.y, qa.z), b = mk3(qb.x, qb.y, qb.z), c = mk3(qc.x, qc.y, qc.z);
      const float da = dot(d, a), db = dot(d, b), dc = dot(d, c);
      if (da > db) return dc > da ? c : a;
      return dc > db ? c : b;
    }
    default:
      return mk3(0.f, 0.f, 0.f);
  }
}

// Support of A - B with B posed in A's frame (minkowski_diff.hpp:21-58):
// pa = s_A(d), pb = T * s_B(-R^T d), both in A's frame.
// Out-of-line copy for the thread-per-pair GJK pass: its lanes diverge over
// shape types and simplex cases, and one shared body keeps the pass's
// instruction footprint small (measured: GJK pass 8 % faster; the warp-wide
// EPA pass keeps the inlined form, which is faster there).
template <int LANES>
__device__ __noinline__ f3 shape_support_outline(const ShapeDev& s, const float4* __restrict__ pool, f3 d,
                                                 const Group<LANES>& g) {
  return shape_support<LANES>(s, pool, d, g);
}

template <int LANES>
struct MinkowskiSupport {
  ShapeDev A, B;
  Pose pose;
  const float4* __restrict__ verts;
  const float4* __restrict__ hull = nullptr;  // walk blocks of kConvexWalk shapes / triangle soup of kTriangle
  Group<LANES> g;
  __device__ __forceinline__ void operator()(f3 d, f3& pa, f3& pb) const {
    if constexpr (LANES < 32) {
      pa = shape_support_outline<LANES>(A, (A.type == kConvexWalk || A.type == kTriangle) ? hull : verts, d, g);
      pb = pose.apply(shape_support_outline<LANES>(B, (B.type == kConvexWalk || B.type == kTriangle) ? hull : verts,
                                                   pose.rotT(-d), g));
    } else {
      pa = shape_support<LANES>(A, verts, d, g);
      pb = pose.apply(shape_support<LANES>(B, verts, pose.rotT(-d), g));
    }
  }
};

}  // namespace fclg
