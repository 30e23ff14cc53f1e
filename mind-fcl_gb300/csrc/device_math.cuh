// Small vector types and the packed records the kernels read and write.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

// The vector helpers below and the FP64 final solve (epa_final_solve) also
// build for the host, where the CPU tests run them.
#define FCLG_HD __host__ __device__ __forceinline__

namespace fclg {

struct f3 {
  float x, y, z;
};
FCLG_HD f3 mk3(float x, float y, float z) { return f3{x, y, z}; }
FCLG_HD f3 operator+(f3 a, f3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
FCLG_HD f3 operator-(f3 a, f3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
FCLG_HD f3 operator-(f3 a) { return mk3(-a.x, -a.y, -a.z); }
FCLG_HD f3 operator*(f3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
FCLG_HD f3 operator*(float s, f3 a) { return mk3(a.x * s, a.y * s, a.z * s); }
FCLG_HD float dot(f3 a, f3 b) { return fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x)); }
FCLG_HD f3 cross(f3 a, f3 b) {
  return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
FCLG_HD float sqn(f3 a) { return dot(a, a); }
FCLG_HD float nrm(f3 a) { return sqrtf(sqn(a)); }
// Leaves a zero vector unchanged (the reference's Eigen normalize()).
__device__ __forceinline__ f3 normalized(f3 a) {
  const float n2 = sqn(a);
  return n2 > 0.f ? a * rsqrtf(n2) : a;
}

struct d3 {
  double x, y, z;
};
FCLG_HD d3 tod(f3 a) { return d3{(double)a.x, (double)a.y, (double)a.z}; }
FCLG_HD d3 operator-(d3 a, d3 b) { return d3{a.x - b.x, a.y - b.y, a.z - b.z}; }
FCLG_HD d3 operator+(d3 a, d3 b) { return d3{a.x + b.x, a.y + b.y, a.z + b.z}; }
FCLG_HD d3 operator*(d3 a, double s) { return d3{a.x * s, a.y * s, a.z * s}; }
FCLG_HD double dot(d3 a, d3 b) { return fma(a.z, b.z, fma(a.y, b.y, a.x * b.x)); }
FCLG_HD d3 cross(d3 a, d3 b) {
  return d3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// Barycentric weights (u, v, w) of the point of triangle (a, b, c) nearest the
// origin (Ericson, Real-Time Collision Detection, 5.1.5), in FP64.
FCLG_HD void closest_bary_origin(d3 a, d3 b, d3 c, double& u, double& v, double& w) {
  const d3 ab = b - a, ac = c - a;
  const d3 ap = a * -1.0, bp = b * -1.0, cp = c * -1.0;
  const double d1 = dot(ab, ap), d2 = dot(ac, ap);
  const double d3v = dot(ab, bp), d4 = dot(ac, bp);
  const double d5 = dot(ab, cp), d6 = dot(ac, cp);
  const double vc = d1 * d4 - d3v * d2, vb = d5 * d2 - d1 * d6, va = d3v * d6 - d5 * d4;
  if (d1 <= 0.0 && d2 <= 0.0) { u = 1; v = 0; w = 0; }
  else if (d3v >= 0.0 && d4 <= d3v) { u = 0; v = 1; w = 0; }
  else if (vc <= 0.0 && d1 >= 0.0 && d3v <= 0.0) { v = d1 / (d1 - d3v); u = 1 - v; w = 0; }
  else if (d6 >= 0.0 && d5 <= d6) { u = 0; v = 0; w = 1; }
  else if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) { w = d2 / (d2 - d6); u = 1 - w; v = 0; }
  else if (va <= 0.0 && (d4 - d3v) >= 0.0 && (d5 - d6) >= 0.0) {
    w = (d4 - d3v) / ((d4 - d3v) + (d5 - d6));
    u = 0;
    v = 1 - w;
  } else {
    const double inv = 1.0 / (va + vb + vc);
    v = vb * inv;
    w = vc * inv;
    u = 1.0 - v - w;
  }
}

// EPA's final closest-face solve in FP64: the point of the final face's
// triangle nearest the origin (closest_bary_origin) and its barycentric
// weights, which interpolate the support points into the witness pair
// (epa.hpp:425-498; when the origin projects into the triangle this is the
// reference's face parameterisation, otherwise its edge / vertex feature).
// Depth is that point's distance from the origin (the reference's
// min_distance_square).  A degenerate triangle falls back to the last support
// pair (cand_pa, cand_pb) like assignPenetrationPair (epa.hpp:340-365).
// wa..wc are the face's Minkowski vertices, pa_a..pa_c their support points on
// shape a.
FCLG_HD void epa_final_solve(f3 wa, f3 wb, f3 wc, f3 pa_a, f3 pa_b, f3 pa_c, f3 cand_pa, f3 cand_pb, f3& p0,
                             f3& p1, float& depth) {
  const d3 a = tod(wa), b = tod(wb), c = tod(wc);
  const d3 ab = b - a, ac = c - a;
  const d3 n = cross(ab, ac);
  if (!(dot(n, n) > 0.0)) {
    p0 = cand_pa;
    p1 = cand_pb;
    depth = nrm(cand_pa - cand_pb);
    return;
  }
  double u, v, w;
  closest_bary_origin(a, b, c, u, v, w);
  const d3 q = (a * u + b * v) + c * w;
  const d3 pa0 = tod(pa_a), pa1 = tod(pa_b), pa2 = tod(pa_c);
  const d3 pb0 = pa0 - a, pb1 = pa1 - b, pb2 = pa2 - c;
  const d3 x0 = (pa0 * u + pa1 * v) + pa2 * w;
  const d3 x1 = (pb0 * u + pb1 * v) + pb2 * w;
  p0 = mk3((float)x0.x, (float)x0.y, (float)x0.z);
  p1 = mk3((float)x1.x, (float)x1.y, (float)x1.z);
  depth = (float)sqrt(dot(q, q));
}

// Shape types: the reference's GJKShapeType values (gjk_shape.h:9-28).
enum : int32_t { kBox = 0, kSphere = 1, kCapsule = 3, kCylinder = 5, kConvex = 100 };
// Decoded form of a convex hull that carries a walk block (never in fclg_shape).
constexpr int32_t kConvexWalk = 101;
// A mesh triangle as a support shape (vofs: its first of three float4 in the
// triangle soup; never in fclg_shape).
constexpr int32_t kTriangle = 102;

// One shape as the kernels use it, decoded from the 32-byte fclg_shape.
// No walk block: the convex support scans every vertex.
constexpr uint32_t kNoWalk = 0xFFFFFFFFu;

struct ShapeDev {
  int32_t type;
  uint32_t vofs, nv;
  float p0, p1, p2;  // box: half extents; sphere: r; capsule/cylinder: r, half length
};

__device__ __forceinline__ ShapeDev load_shape(const int4* __restrict__ shapes, uint32_t i) {
  const int4 h = __ldg(shapes + 2 * (size_t)i);
  const float4 p = __ldg(reinterpret_cast<const float4*>(shapes) + 2 * (size_t)i + 1);
  ShapeDev s;
  s.type = h.x;
  s.vofs = (uint32_t)h.y;
  s.nv = (uint32_t)h.z;
  if (s.type == kBox) {
    s.p0 = 0.5f * p.x; s.p1 = 0.5f * p.y; s.p2 = 0.5f * p.z;
  } else {
    s.p0 = p.x; s.p1 = 0.5f * p.y; s.p2 = 0.f;
  }
  return s;
}

// load_shape for one-lane groups: a hull with a walk block (walk_tab: per-shape
// first entry or kNoWalk; null for none) decodes as kConvexWalk with vofs = the
// block's first entry.
__device__ __forceinline__ ShapeDev load_shape(const int4* __restrict__ shapes, const uint32_t* __restrict__ walk_tab,
                                               uint32_t i) {
  ShapeDev s = load_shape(shapes, i);
  if (walk_tab && s.type == kConvex) {
    const uint32_t w = __ldg(walk_tab + i);
    if (w != kNoWalk) {
      s.type = kConvexWalk;
      s.vofs = w;
    }
  }
  return s;
}

// Pose of shape b in shape a's frame (the reference's MinkowskiDiff::toshape0).
struct Pose {
  float r[9];
  f3 t;
  __device__ __forceinline__ f3 rot(f3 v) const {
    return mk3(fmaf(r[2], v.z, fmaf(r[1], v.y, r[0] * v.x)), fmaf(r[5], v.z, fmaf(r[4], v.y, r[3] * v.x)),
               fmaf(r[8], v.z, fmaf(r[7], v.y, r[6] * v.x)));
  }
  __device__ __forceinline__ f3 rotT(f3 v) const {
    return mk3(fmaf(r[6], v.z, fmaf(r[3], v.y, r[0] * v.x)), fmaf(r[7], v.z, fmaf(r[4], v.y, r[1] * v.x)),
               fmaf(r[8], v.z, fmaf(r[5], v.y, r[2] * v.x)));
  }
  __device__ __forceinline__ f3 apply(f3 v) const { return rot(v) + t; }
};

struct PairDev {
  uint32_t a, b;
  Pose pose;
};

__device__ __forceinline__ PairDev load_pair(const float4* __restrict__ pairs, uint32_t i) {
  const float4 q0 = __ldg(pairs + 4 * (size_t)i + 0);
  const float4 q1 = __ldg(pairs + 4 * (size_t)i + 1);
  const float4 q2 = __ldg(pairs + 4 * (size_t)i + 2);
  const float4 q3 = __ldg(pairs + 4 * (size_t)i + 3);
  PairDev p;
  p.a = __float_as_uint(q0.x);
  p.b = __float_as_uint(q0.y);
  p.pose.r[0] = q0.z; p.pose.r[1] = q0.w;
  p.pose.r[2] = q1.x; p.pose.r[3] = q1.y; p.pose.r[4] = q1.z; p.pose.r[5] = q1.w;
  p.pose.r[6] = q2.x; p.pose.r[7] = q2.y; p.pose.r[8] = q2.z;
  p.pose.t = mk3(q2.w, q3.x, q3.y);
  return p;
}

// Status word of a result: bits 0-7 GJK_Status, bits 8-15 EPA_Status + 1.
enum : int32_t { kGjkIntersect = 0, kGjkSeparated = 1, kGjkNoProgress = 2, kGjkIterLimit = 3, kGjkFailed = 4 };
// Result status bit: the boolean came from MPR (bits 0-7 then hold Intersect / Separated).
constexpr int32_t kStatusMpr = 1 << 16;
// Result status bit: the answer came from a closed-form sphere-pair solver.
constexpr int32_t kStatusAnalytic = 1 << 17;
// Result status bit: MPR directed penetration ran (bits 8-15 its status + 1).
constexpr int32_t kStatusDirected = 1 << 18;
// Result status bit: MPR incremental penetration ran (bits 8-15 its status + 1).
constexpr int32_t kStatusIncremental = 1 << 19;
enum : int32_t { kEpaFailed = 0, kEpaOK = 1, kEpaTouching = 2, kEpaIterLimit = 3, kEpaMallocFailed = 4 };

// 48-byte fclg_result written as three float4 stores.
__device__ __forceinline__ void store_result(float4* __restrict__ out, uint32_t i, float dist, f3 n, f3 pa, f3 pb,
                                             int32_t status, uint32_t iters, bool collide, bool ok) {
  const uint32_t tail = (iters > 0xFFFFu ? 0xFFFFu : iters) | ((collide ? 1u : 0u) << 16) | ((ok ? 1u : 0u) << 24);
  out[3 * (size_t)i + 0] = make_float4(dist, n.x, n.y, n.z);
  out[3 * (size_t)i + 1] = make_float4(pa.x, pa.y, pa.z, pb.x);
  out[3 * (size_t)i + 2] = make_float4(pb.y, pb.z, __int_as_float(status), __uint_as_float(tail));
}

// Scalar parameters of a query batch (GJKSolver fields, gjk_solver.h:122-163).
struct QueryParams {
  float gjk_tol;
  float epa_tol;
  int gjk_max_iter;
  int epa_max_iter;
  int epa_max_faces;
  int want_distance;  // 1: signed distance (GJK distance / EPA); 0: boolean only
  int use_mpr;        // boolean collide: MPR first, GJK when MPR fails
  int analytic;       // collide: closed-form solvers for sphere pairs
  int directed;       // collide with MPR directed penetration along BatchArgs::guess (directed_pass.cu)
  int incremental;    // directed_pass: the incremental penetration from BatchArgs::guess as the hint
  int want_epa;       // run EPA on overlapping pairs
  int warm_probe;     // learned starts: supports the boolean phase gets to certify separation (0: no limit)
  float warm_gap;     // learned starts: duality gap that certifies the distance (0: the reference's stop)
};

}  // namespace fclg
