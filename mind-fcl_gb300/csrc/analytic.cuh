// Closed-form contacts for sphere pairs, the solvers fcl::collide dispatches
// to instead of MPR / GJK+EPA (ShapeIntersectIndepImpl specialisations,
// gjk_solver-inl.h:209-218), in FP32, one thread per pair:
//   sphere-sphere    primitive_shape_algorithm/sphere_sphere-inl.h:48-66
//   sphere-capsule   primitive_shape_algorithm/sphere_capsule-inl.h:49-63, 70-100
//   sphere-box       primitive_shape_algorithm/sphere_box-inl.h:59-172
//   sphere-cylinder  primitive_shape_algorithm/sphere_cylinder-inl.h:60-201
//   box-box          primitive_shape_algorithm/box_box-inl.h:52-212, 214-802
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
  float separation;  // when not hit: centre-based separation (sphere pairs), the gap along the
                     // separating axis found, unnormalised for edge axes (box pairs)
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

// ---------------------------------------------------------------- box-box --
// boxBox2 with box 1 axis-aligned at the origin (half extents A) and box 2
// (half extents B) posed by X: the 15 separating-axis tests, then the
// edge-edge point or the clipped face manifold culled to four points; out
// holds the first contact of maximal depth, which a one-contact fcl::collide
// reports (shape_pair_intersect-inl.h:92-104).  Out of line: the pass's other
// shapes keep their registers.

// intersectRectQuad2 (box_box-inl.h:76-137): clip quad q (4 points) by the
// lines x = -h0, x = h0, y = -h1, y = h1; the result (at most 8) in ret.
__device__ __forceinline__ int clip_rect_quad(float h0, float h1, const float q0[8], float ret[16]) {
  float bufA[16], bufB[16];
#pragma unroll
  for (int k = 0; k < 8; ++k) bufA[k] = q0[k];
  float* q = bufA;
  float* r = bufB;
  int nq = 4;
  for (int dir = 0; dir <= 1; ++dir) {
    const float h = dir ? h1 : h0;
    for (int sign = -1; sign <= 1; sign += 2) {
      int nr = 0;
      for (int i = 0; i < nq; ++i) {
        const float* cur = q + 2 * i;
        const float* nxt = q + 2 * (i + 1 < nq ? i + 1 : 0);
        const bool in_cur = (float)sign * cur[dir] < h;
        if (in_cur) {
          r[2 * nr] = cur[0];
          r[2 * nr + 1] = cur[1];
          if (++nr == 8) {
            for (int k = 0; k < 16; ++k) ret[k] = r[k];
            return 8;
          }
        }
        if (in_cur != ((float)sign * nxt[dir] < h)) {
          r[2 * nr + 1 - dir] =
              cur[1 - dir] + (nxt[1 - dir] - cur[1 - dir]) / (nxt[dir] - cur[dir]) * ((float)sign * h - cur[dir]);
          r[2 * nr + dir] = (float)sign * h;
          if (++nr == 8) {
            for (int k = 0; k < 16; ++k) ret[k] = r[k];
            return 8;
          }
        }
      }
      float* t = q;
      q = r;
      r = t;
      nq = nr;
    }
  }
  for (int k = 0; k < 2 * nq; ++k) ret[k] = q[k];
  return nq;
}

// cullPoints2 (box_box-inl.h:139-212): m of the n points, starting at i0, then
// the free point whose angle about the centroid is nearest A[i0] + j 2 pi / m.
__device__ __forceinline__ void cull_points(int n, const float p[16], int m, int i0, int iret[8]) {
  float cx, cy;
  if (n == 1) {
    cx = p[0];
    cy = p[1];
  } else if (n == 2) {
    cx = 0.5f * (p[0] + p[2]);
    cy = 0.5f * (p[1] + p[3]);
  } else {
    float a = 0.f, q;
    cx = cy = 0.f;
    for (int i = 0; i < n - 1; ++i) {
      q = p[i * 2] * p[i * 2 + 3] - p[i * 2 + 2] * p[i * 2 + 1];
      a += q;
      cx += q * (p[i * 2] + p[i * 2 + 2]);
      cy += q * (p[i * 2 + 1] + p[i * 2 + 3]);
    }
    q = p[n * 2 - 2] * p[1] - p[0] * p[n * 2 - 1];
    a = fabsf(a + q) > 1.1920929e-07f ? 1.f / (3.f * (a + q)) : 1e18f;
    cx = a * (cx + q * (p[n * 2 - 2] + p[0]));
    cy = a * (cy + q * (p[n * 2 - 1] + p[1]));
  }
  float ang[8];
  unsigned avail = 0;
  for (int i = 0; i < n; ++i) {
    ang[i] = atan2f(p[i * 2 + 1] - cy, p[i * 2] - cx);
    avail |= 1u << i;
  }
  avail &= ~(1u << i0);
  iret[0] = i0;
  const float pi = 3.14159265358979f;
  for (int j = 1; j < m; ++j) {
    float a = (float)j * (2.f * pi / (float)m) + ang[i0];
    if (a > pi) a -= 2.f * pi;
    float maxdiff = 1e9f;
    iret[j] = i0;
    for (int i = 0; i < n; ++i) {
      if (!((avail >> i) & 1u)) continue;
      float diff = fabsf(ang[i] - a);
      if (diff > pi) diff = 2.f * pi - diff;
      if (diff < maxdiff) {
        maxdiff = diff;
        iret[j] = i;
      }
    }
    avail &= ~(1u << iret[j]);
  }
}

static __device__ __noinline__ AnalyticContact box_box(f3 A, f3 B, const Pose& X) {
  AnalyticContact out;
  out.hit = false;
  out.separation = 0.f;
  out.depth = 0.f;
  out.normal = mk3(0.f, 0.f, 0.f);
  out.pos = mk3(0.f, 0.f, 0.f);
  const float a[3] = {A.x, A.y, A.z}, b[3] = {B.x, B.y, B.z};
  const float p[3] = {X.t.x, X.t.y, X.t.z};  // = pp: box 1 is the frame
  float Q[3][3];
#pragma unroll
  for (int i = 0; i < 9; ++i) Q[i / 3][i % 3] = fabsf(X.r[i]);
  auto R = [&](int i, int j) { return X.r[3 * i + j]; };
  float s = -3.402823466e38f;
  int code = 0, best_col = -1, invert = 0;
  float nC[3] = {0.f, 0.f, 0.f};
  for (int i = 0; i < 3; ++i) {
    const float tmp = p[i];
    const float s2 = fabsf(tmp) - (((Q[i][0] * b[0] + Q[i][1] * b[1]) + Q[i][2] * b[2]) + a[i]);
    if (s2 > 0.f) { out.separation = s2; return out; }
    if (s2 > s) { s = s2; best_col = i; invert = tmp < 0.f; code = i + 1; }
  }
  for (int j = 0; j < 3; ++j) {
    const float tmp = (R(0, j) * p[0] + R(1, j) * p[1]) + R(2, j) * p[2];
    const float s2 = fabsf(tmp) - (((Q[0][j] * a[0] + Q[1][j] * a[1]) + Q[2][j] * a[2]) + b[j]);
    if (s2 > 0.f) { out.separation = s2; return out; }
    if (s2 > s) { s = s2; best_col = j; invert = tmp < 0.f; code = j + 4; }
  }
  const float eps = 1.1920929e-07f;
  const float scale = fmaxf(fmaxf(fmaxf(fmaxf(a[0], a[1]), a[2]), fmaxf(fmaxf(b[0], b[1]), b[2])), 1.f) * 10.f * eps;
#pragma unroll
  for (int i = 0; i < 9; ++i) Q[i / 3][i % 3] += scale;
  for (int i = 0; i < 3; ++i) {
    const int c1 = (i + 1) % 3, c2 = (i + 2) % 3;
    const int lo = i == 0 ? 1 : 0, hi = i == 2 ? 1 : 2;
    for (int j = 0; j < 3; ++j) {
      const int jlo = j == 0 ? 1 : 0, jhi = j == 2 ? 1 : 2;
      const float tmp = p[c2] * R(c1, j) - p[c1] * R(c2, j);
      const float s2 = fabsf(tmp) - (a[lo] * Q[hi][j] + a[hi] * Q[lo][j] + b[jlo] * Q[i][jhi] + b[jhi] * Q[i][jlo]);
      if (s2 > 0.f) { out.separation = s2; return out; }
      float n[3];
      n[i] = 0.f;
      n[c1] = -R(c2, j);
      n[c2] = R(c1, j);
      const float l = sqrtf((n[0] * n[0] + n[1] * n[1]) + n[2] * n[2]);
      if (l > eps) {
        const float s2n = s2 / l;
        if (s2n * 1.05f > s) {
          s = s2n;
          best_col = -1;
          nC[0] = n[0] / l;
          nC[1] = n[1] / l;
          nC[2] = n[2] / l;
          invert = tmp < 0.f;
          code = 7 + 3 * i + j;
        }
      }
    }
  }
  f3 normal;
  if (best_col == -1) normal = mk3(nC[0], nC[1], nC[2]);
  else if (code <= 3) normal = mk3(best_col == 0 ? 1.f : 0.f, best_col == 1 ? 1.f : 0.f, best_col == 2 ? 1.f : 0.f);
  else normal = mk3(R(0, best_col), R(1, best_col), R(2, best_col));
  if (invert) normal = -normal;
  out.hit = true;
  out.normal = normal;
  out.depth = -s;
  out.pos = X.t * 0.5f;
  auto col2 = [&](int c) { return mk3(R(0, c), R(1, c), R(2, c)); };
  const float nv[3] = {normal.x, normal.y, normal.z};
  if (code > 6) {
    // edge-edge (box_box-inl.h:555-594)
    f3 pa = mk3(0.f, 0.f, 0.f);
    pa.x += a[0] * (nv[0] > 0.f ? 1.f : -1.f);
    pa.y += a[1] * (nv[1] > 0.f ? 1.f : -1.f);
    pa.z += a[2] * (nv[2] > 0.f ? 1.f : -1.f);
    f3 pb = X.t;
    for (int j = 0; j < 3; ++j) pb = pb + col2(j) * (b[j] * (dot(col2(j), normal) > 0.f ? -1.f : 1.f));
    const int ia = (code - 7) / 3;
    const f3 ua = mk3(ia == 0 ? 1.f : 0.f, ia == 1 ? 1.f : 0.f, ia == 2 ? 1.f : 0.f);
    const f3 ub = col2((code - 7) % 3);
    const f3 pd = pb - pa;
    const float uaub = dot(ua, ub), q1 = dot(ua, pd), q2 = -dot(ub, pd);
    float d = 1.f - uaub * uaub, alpha = 0.f, beta = 0.f;
    if (d > 0.0001f) {
      d = 1.f / d;
      alpha = (q1 + uaub * q2) * d;
      beta = (uaub * q1 + q2) * d;
    }
    out.pos = ((pa + ua * alpha) + (pb + ub * beta)) * 0.5f;
    return out;
  }
  // face-something (box_box-inl.h:595-800): reference face on box 1 for codes 1-3
  const bool ref1 = code <= 3;
  auto cola = [&](int c) { return ref1 ? mk3(c == 0 ? 1.f : 0.f, c == 1 ? 1.f : 0.f, c == 2 ? 1.f : 0.f) : col2(c); };
  auto colb = [&](int c) { return ref1 ? col2(c) : mk3(c == 0 ? 1.f : 0.f, c == 1 ? 1.f : 0.f, c == 2 ? 1.f : 0.f); };
  const f3 Pa = ref1 ? mk3(0.f, 0.f, 0.f) : X.t, Pb = ref1 ? X.t : mk3(0.f, 0.f, 0.f);
  const float* Sa = ref1 ? a : b;
  const float* Sb = ref1 ? b : a;
  const f3 normal2 = ref1 ? normal : -normal;
  const float nr[3] = {dot(colb(0), normal2), dot(colb(1), normal2), dot(colb(2), normal2)};
  const float anr[3] = {fabsf(nr[0]), fabsf(nr[1]), fabsf(nr[2])};
  int lanr, a1, a2;
  if (anr[1] > anr[0]) {
    if (anr[1] > anr[2]) { a1 = 0; lanr = 1; a2 = 2; }
    else { a1 = 0; a2 = 1; lanr = 2; }
  } else {
    if (anr[0] > anr[2]) { lanr = 0; a1 = 1; a2 = 2; }
    else { a1 = 0; a2 = 1; lanr = 2; }
  }
  const f3 center = nr[lanr] < 0.f ? (Pb - Pa) + colb(lanr) * Sb[lanr] : (Pb - Pa) - colb(lanr) * Sb[lanr];
  const int codeN = ref1 ? code - 1 : code - 4;
  const int code1 = codeN == 0 ? 1 : 0, code2 = codeN == 2 ? 1 : 2;
  const float c1 = dot(cola(code1), center), c2 = dot(cola(code2), center);
  float m11 = dot(colb(a1), cola(code1)), m12 = dot(colb(a2), cola(code1));
  float m21 = dot(colb(a1), cola(code2)), m22 = dot(colb(a2), cola(code2));
  float quad[8];
  {
    const float k1 = m11 * Sb[a1], k2 = m21 * Sb[a1], k3 = m12 * Sb[a2], k4 = m22 * Sb[a2];
    quad[0] = c1 - k1 - k3;
    quad[1] = c2 - k2 - k4;
    quad[2] = c1 - k1 + k3;
    quad[3] = c2 - k2 + k4;
    quad[4] = c1 + k1 + k3;
    quad[5] = c2 + k2 + k4;
    quad[6] = c1 + k1 - k3;
    quad[7] = c2 + k2 - k4;
  }
  float ret[16];
  const int n_int = clip_rect_quad(Sa[code1], Sa[code2], quad, ret);
  if (n_int < 1) return out;
  const float det1 = 1.f / (m11 * m22 - m12 * m21);
  m11 *= det1;
  m12 *= det1;
  m21 *= det1;
  m22 *= det1;
  f3 pts[8];
  float dep[8];
  int cnum = 0;
  for (int j = 0; j < n_int; ++j) {
    const float k1 = m22 * (ret[j * 2] - c1) - m12 * (ret[j * 2 + 1] - c2);
    const float k2 = -m21 * (ret[j * 2] - c1) + m11 * (ret[j * 2 + 1] - c2);
    const f3 pt = center + colb(a1) * k1 + colb(a2) * k2;
    const float dj = Sa[codeN] - dot(normal2, pt);
    if (dj >= 0.f) {
      pts[cnum] = pt;
      dep[cnum] = dj;
      ret[cnum * 2] = ret[j * 2];
      ret[cnum * 2 + 1] = ret[j * 2 + 1];
      cnum++;
    }
  }
  if (cnum < 1) return out;
  int iret[8] = {0, 1, 2, 3, 4, 5, 6, 7};
  int m = cnum < 4 ? cnum : 4;
  if (cnum > m) {
    int i1 = 0;
    for (int i = 1; i < cnum; ++i)
      if (dep[i] > dep[i1]) i1 = i;
    cull_points(cnum, ret, m, i1, iret);
    cnum = m;
  }
  int k = iret[0];
  for (int j = 1; j < cnum; ++j)
    if (dep[iret[j]] > dep[k]) k = iret[j];
  const f3 half = normal * (dep[k] * 0.5f);
  out.depth = dep[k];
  out.pos = ref1 ? pts[k] + Pa + half : pts[k] + Pa - half;
  return out;
}

// True when (a, b) is a pair with a closed-form solver (sphere pairs, box-box); fills out.
__device__ __forceinline__ bool analytic_contact(const ShapeDev& A, const ShapeDev& B, const Pose& pose,
                                                 AnalyticContact& out) {
  const bool sa = A.type == kSphere, sb = B.type == kSphere;
  if (A.type == kBox && B.type == kBox) {
    out = box_box(mk3(A.p0, A.p1, A.p2), mk3(B.p0, B.p1, B.p2), pose);
    return true;
  }
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
