// Closed-form contacts for sphere pairs, the solvers fcl::collide dispatches
// to instead of MPR / GJK+EPA (ShapeIntersectIndepImpl specialisations,
// gjk_solver-inl.h:209-218), in FP32, one thread per pair:
//   sphere-sphere    primitive_shape_algorithm/sphere_sphere-inl.h:48-66
//   sphere-capsule   primitive_shape_algorithm/sphere_capsule-inl.h:49-63, 70-100
//   sphere-box       primitive_shape_algorithm/sphere_box-inl.h:59-172
//   sphere-cylinder  primitive_shape_algorithm/sphere_cylinder-inl.h:60-201
// Reversed pairs run the same solver with the shapes swapped and flip the
// normal (gjk_solver-inl.h:190-201).  Shape a sits at the origin, shape b at
// the pair's pose; the contact normal is the escape direction of b.
#pragma once
#include "device_math.cuh"

namespace fclg {

struct AnalyticContact {
  bool hit;
  f3 normal, pos;
  float depth;
  float separation;  // when not hit: centre-based separation of the pair
};

// The reference's noise floor for these solvers: 16 eps of the scalar type.
constexpr float kAnalyticEps = 16.f * 1.1920929e-07f;

__device__ __forceinline__ f3 seg_closest(f3 p, f3 s1, f3 s2) {
  const f3 v = s2 - s1, w = p - s1;
  const float c1 = dot(w, v), c2 = dot(v, v);
  if (c1 <= 0.f) return s1;
  if (c2 <= c1) return s2;
  return s1 + v * (c1 / c2);
}

// Sphere (radius rs) centred at c in frame F; the other shape posed by X in F.
// Returns c in the other shape's frame.
__device__ __forceinline__ f3 to_local(const Pose& X, f3 c) { return X.rotT(c - X.t); }

__device__ __forceinline__ AnalyticContact sphere_sphere(float r1, float r2, f3 c2) {
  AnalyticContact a;
  const float len = nrm(c2);
  a.hit = !(len > r1 + r2);
  a.separation = len - (r1 + r2);
  a.normal = len > 0.f ? c2 * (1.f / len) : c2;
  a.pos = c2 * (r1 / (r1 + r2));
  a.depth = r1 + r2 - len;
  return a;
}

__device__ __forceinline__ AnalyticContact sphere_capsule(float rs, float rc, float lz, const Pose& X, f3 c) {
  AnalyticContact a;
  const f3 s_c = to_local(X, c);
  const f3 sp = seg_closest(s_c, mk3(0.f, 0.f, 0.5f * lz), mk3(0.f, 0.f, -0.5f * lz));
  const f3 diff = s_c - sp;
  const float distance = nrm(diff) - rs - rc;
  a.hit = !(distance > 0.f);
  a.separation = distance;
  const f3 ln = -normalized(diff);
  a.normal = X.rot(ln);
  a.pos = X.apply(sp + ln * distance);
  a.depth = -distance;
  return a;
}

__device__ __forceinline__ AnalyticContact sphere_box(float r, f3 half, const Pose& X, f3 c) {
  AnalyticContact a;
  const f3 p = to_local(X, c);
  f3 nb = p;
  bool clamped = false;
  if (p.x < -half.x) { clamped = true; nb.x = -half.x; }
  if (p.x > half.x) { clamped = true; nb.x = half.x; }
  if (p.y < -half.y) { clamped = true; nb.y = -half.y; }
  if (p.y > half.y) { clamped = true; nb.y = half.y; }
  if (p.z < -half.z) { clamped = true; nb.z = -half.z; }
  if (p.z > half.z) { clamped = true; nb.z = half.z; }
  const f3 cn = nb - p;
  const float sq = sqn(cn);
  a.hit = !(sq > r * r);
  a.separation = sqrtf(sq) - r;
  f3 n, pp;
  if (clamped && sq > kAnalyticEps * kAnalyticEps) {
    const float d = sqrtf(sq);
    n = cn * (1.f / d);
    a.depth = r - d;
    pp = nb + n * (a.depth * 0.5f);
  } else {
    const float dx = p.x >= 0.f ? half.x - p.x : p.x + half.x;
    const float dy = p.y >= 0.f ? half.y - p.y : p.y + half.y;
    const float dz = p.z >= 0.f ? half.z - p.z : p.z + half.z;
    float md = INFINITY;
    int axis = -1;
    if (dx + kAnalyticEps < md) { md = dx; axis = 0; }
    if (dy + kAnalyticEps < md) { md = dy; axis = 1; }
    if (dz + kAnalyticEps < md) { md = dz; axis = 2; }
    n = mk3(0.f, 0.f, 0.f);
    if (axis == 0) n.x = p.x >= 0.f ? -1.f : 1.f;
    else if (axis == 1) n.y = p.y >= 0.f ? -1.f : 1.f;
    else n.z = p.z >= 0.f ? -1.f : 1.f;
    a.depth = md + r;
    pp = p + n * ((r - md) * 0.5f);
  }
  a.normal = X.rot(n);
  a.pos = X.apply(pp);
  return a;
}

__device__ __forceinline__ AnalyticContact sphere_cylinder(float rs, float rc, float lz, const Pose& X, f3 c) {
  AnalyticContact a;
  const f3 p = to_local(X, c);
  f3 nb = p;
  bool outside = false;
  const float hh = 0.5f * lz;
  if (p.z > hh) { outside = true; nb.z = hh; }
  else if (p.z < -hh) { outside = true; nb.z = -hh; }
  const float sqxy = p.x * p.x + p.y * p.y;
  if (sqxy > rc * rc) {
    outside = true;
    const float k = rc / sqrtf(sqxy);
    nb.x = p.x * k;
    nb.y = p.y * k;
  }
  const f3 sn = nb - p;
  const float sq = sqn(sn);
  a.hit = !(sq > rs * rs);
  a.separation = sqrtf(sq) - rs;
  f3 n, pp;
  if (outside && sq > kAnalyticEps * kAnalyticEps) {
    const float d = sqrtf(sq);
    n = sn * (1.f / d);
    a.depth = rs - d;
    pp = nb + n * (a.depth * 0.5f);
  } else {
    const float face = p.z >= 0.f ? hh - p.z : p.z + hh;
    const float dxy = sqrtf(p.x * p.x + p.y * p.y);
    const float barrel = rc - dxy;
    if (barrel < face - kAnalyticEps) {
      if (dxy > kAnalyticEps) {
        n = mk3(-p.x / dxy, -p.y / dxy, 0.f);
        a.depth = rs + barrel;
      } else {
        n = mk3(-1.f, 0.f, 0.f);
        a.depth = rs + rc;
      }
      pp = p + n * ((rs - barrel) * 0.5f);
    } else {
      n = mk3(0.f, 0.f, p.z >= 0.f ? -1.f : 1.f);
      a.depth = face + rs;
      pp = p + n * ((rs - face) * 0.5f);
    }
  }
  a.normal = X.rot(n);
  a.pos = X.apply(pp);
  return a;
}

// True when (a, b) is a sphere pair with a closed-form solver; fills out.
__device__ __forceinline__ bool analytic_contact(const ShapeDev& A, const ShapeDev& B, const Pose& pose,
                                                 AnalyticContact& out) {
  const bool sa = A.type == kSphere, sb = B.type == kSphere;
  if (!sa && !sb) return false;
  if (sa && sb) {
    out = sphere_sphere(A.p0, B.p0, pose.t);
    return true;
  }
  const ShapeDev& o = sa ? B : A;
  if (o.type != kCapsule && o.type != kBox && o.type != kCylinder) return false;
  // ShapeDev holds box half extents and capsule / cylinder half lengths
  const float lz = 2.f * o.p1;
  if (sa) {
    const f3 c = mk3(0.f, 0.f, 0.f);
    if (o.type == kCapsule) out = sphere_capsule(A.p0, o.p0, lz, pose, c);
    else if (o.type == kBox) out = sphere_box(A.p0, mk3(o.p0, o.p1, o.p2), pose, c);
    else out = sphere_cylinder(A.p0, o.p0, lz, pose, c);
    return true;
  }
  Pose I;
#pragma unroll
  for (int k = 0; k < 9; ++k) I.r[k] = (k % 4 == 0) ? 1.f : 0.f;
  I.t = mk3(0.f, 0.f, 0.f);
  if (o.type == kCapsule) out = sphere_capsule(B.p0, o.p0, lz, I, pose.t);
  else if (o.type == kBox) out = sphere_box(B.p0, mk3(o.p0, o.p1, o.p2), I, pose.t);
  else out = sphere_cylinder(B.p0, o.p0, lz, I, pose.t);
  out.normal = -out.normal;
  return true;
}

}  // namespace fclg
