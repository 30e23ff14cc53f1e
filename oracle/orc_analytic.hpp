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
//   boxBoxIntersect          primitive_shape_algorithm/box_box-inl.h:52-212, 214-802, 823-839
#pragma once
#include <cstring>

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

// ---------------------------------------------------------------- box-box --
// lineClosestApproach, box_box-inl.h:52-74: parameters of the closest points
// of the lines pa + alpha ua and pb + beta ub (0, 0 when nearly parallel).
inline void lineClosestApproach(const V3& pa, const V3& ua, const V3& pb, const V3& ub, double& alpha,
                                double& beta) {
  const V3 p = pb - pa;
  const double uaub = dot(ua, ub), q1 = dot(ua, p), q2 = -dot(ub, p);
  double d = 1 - uaub * uaub;
  if (d <= (double)0.0001f) {
    alpha = beta = 0;
    return;
  }
  d = 1 / d;
  alpha = (q1 + uaub * q2) * d;
  beta = (uaub * q1 + q2) * d;
}

// intersectRectQuad2, box_box-inl.h:76-137: clips the quadrilateral p (4 x,y
// points) against the rectangle |x| < h[0], |y| < h[1], one edge line at a
// time (x = -h0, x = +h0, y = -h1, y = +h1); returns the clipped polygon's
// point count (at most 8) in ret.
inline int intersectRectQuad2(const double h[2], const double p[8], double ret[16]) {
  double bufA[16], bufB[16];
  std::memcpy(bufA, p, 8 * sizeof(double));
  double* q = bufA;
  double* r = bufB;
  int nq = 4, nr = 0;
  for (int dir = 0; dir <= 1; ++dir)
    for (int sign = -1; sign <= 1; sign += 2) {
      nr = 0;
      for (int i = 0; i < nq; ++i) {
        const double* cur = q + 2 * i;
        const double* nxt = q + 2 * ((i + 1) % nq);
        const bool in_cur = sign * cur[dir] < h[dir];
        if (in_cur) {
          r[2 * nr] = cur[0];
          r[2 * nr + 1] = cur[1];
          if (++nr == 8) goto done;
        }
        if (in_cur != (sign * nxt[dir] < h[dir])) {
          r[2 * nr + 1 - dir] = cur[1 - dir] + (nxt[1 - dir] - cur[1 - dir]) / (nxt[dir] - cur[dir]) *
                                                   (sign * h[dir] - cur[dir]);
          r[2 * nr + dir] = sign * h[dir];
          if (++nr == 8) goto done;
        }
      }
      std::swap(q, r);
      nq = nr;
    }
  std::memcpy(ret, q, (size_t)nq * 2 * sizeof(double));
  return nq;
done:
  std::memcpy(ret, r, 16 * sizeof(double));
  return 8;
}

// cullPoints2, box_box-inl.h:139-212: keeps m of the n polygon points p,
// starting with point i0, then the available point whose angle about the
// polygon's centroid is nearest to A[i0] + j 2 pi / m, j = 1 .. m-1.
inline void cullPoints2(int n, const double p[], int m, int i0, int iret[]) {
  double cx, cy;
  if (n == 1) {
    cx = p[0];
    cy = p[1];
  } else if (n == 2) {
    cx = 0.5 * (p[0] + p[2]);
    cy = 0.5 * (p[1] + p[3]);
  } else {
    double a = 0, q;
    cx = cy = 0;
    for (int i = 0; i < n - 1; ++i) {
      q = p[i * 2] * p[i * 2 + 3] - p[i * 2 + 2] * p[i * 2 + 1];
      a += q;
      cx += q * (p[i * 2] + p[i * 2 + 2]);
      cy += q * (p[i * 2 + 1] + p[i * 2 + 3]);
    }
    q = p[n * 2 - 2] * p[1] - p[0] * p[n * 2 - 1];
    if (std::abs(a + q) > std::numeric_limits<double>::epsilon()) a = 1 / (3 * (a + q));
    else a = (double)1e18f;
    cx = a * (cx + q * (p[n * 2 - 2] + p[0]));
    cy = a * (cy + q * (p[n * 2 - 1] + p[1]));
  }
  double ang[8];
  for (int i = 0; i < n; ++i) ang[i] = std::atan2(p[i * 2 + 1] - cy, p[i * 2] - cx);
  bool avail[8];
  for (int i = 0; i < n; ++i) avail[i] = true;
  avail[i0] = false;
  iret[0] = i0;
  const double pi = 3.141592653589793238462643383279502884197169399375105820974944592;
  for (int j = 1; j < m; ++j) {
    double a = j * (2 * pi / m) + ang[i0];
    if (a > pi) a -= 2 * pi;
    double maxdiff = 1e9;
    iret[j] = i0;
    for (int i = 0; i < n; ++i) {
      if (!avail[i]) continue;
      double diff = std::abs(ang[i] - a);
      if (diff > pi) diff = 2 * pi - diff;
      if (diff < maxdiff) {
        maxdiff = diff;
        iret[j] = i;
      }
    }
    avail[iret[j]] = false;
  }
}

struct BoxContact {
  V3 normal, pos;
  double depth;
};

// boxBox2, box_box-inl.h:214-802, for box 1 (full sides side1) posed by
// (R1, T1) and box 2 by (R2, T2): the 15 separating-axis tests (face axes of
// either box, then the 9 edge-edge axes with Q padded by the rounding margin
// and a 5 % preference for face axes), then either the edge-edge contact
// point or the face clip (incident face of the other box clipped by the
// reference face, penetrating points kept, culled to maxc).  Returns the
// contact count; code = the axis (1-15), 0 when separated.  separation = the
// gap along the separating axis found (unnormalised for edge axes).
inline int boxBox2(const V3& side1, const double R1[9], const V3& T1, const V3& side2, const double R2[9],
                   const V3& T2, V3& normal, double& depth, int& code, int maxc, BoxContact* contacts,
                   double& separation) {
  auto r1 = [&](int r, int c) { return R1[3 * r + c]; };
  auto r2 = [&](int r, int c) { return R2[3 * r + c]; };
  auto col1 = [&](int c) { return V3(R1[c], R1[3 + c], R1[6 + c]); };
  auto col2 = [&](int c) { return V3(R2[c], R2[3 + c], R2[6 + c]); };
  const double fudge_factor = 1.05;
  const V3 p = T2 - T1;
  const V3 pp(dot(col1(0), p), dot(col1(1), p), dot(col1(2), p));  // R1^T p
  const V3 A = side1 * 0.5, B = side2 * 0.5;
  double R[3][3], Q[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      R[i][j] = (r1(0, i) * r2(0, j) + r1(1, i) * r2(1, j)) + r1(2, i) * r2(2, j);  // (R1^T R2)(i, j)
      Q[i][j] = std::abs(R[i][j]);
    }
  double s = -std::numeric_limits<double>::max();
  int best_col = -1, best_box = 0, invert = 0;
  V3 normalC;
  code = 0;
  separation = 0;
  // face axes of box 1 (codes 1-3) and of box 2 (codes 4-6)
  for (int i = 0; i < 3; ++i) {
    const double tmp = pp[i];
    const double s2 = std::abs(tmp) - (((Q[i][0] * B[0] + Q[i][1] * B[1]) + Q[i][2] * B[2]) + A[i]);
    if (s2 > 0) { separation = s2; code = 0; return 0; }
    if (s2 > s) { s = s2; best_col = i; best_box = 1; invert = tmp < 0; code = i + 1; }
  }
  for (int j = 0; j < 3; ++j) {
    const double tmp = dot(col2(j), p);
    const double s2 = std::abs(tmp) - (((Q[0][j] * A[0] + Q[1][j] * A[1]) + Q[2][j] * A[2]) + B[j]);
    if (s2 > 0) { separation = s2; code = 0; return 0; }
    if (s2 > s) { s = s2; best_col = j; best_box = 2; invert = tmp < 0; code = j + 4; }
  }
  // pad Q against parallel-edge cross products that round to non-zero
  const double eps = std::numeric_limits<double>::epsilon();
  const double scale = std::max(std::max(std::max(std::max(A[0], A[1]), A[2]), std::max(std::max(B[0], B[1]), B[2])),
                                1.0) * 10.0 * eps;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) Q[i][j] += scale;
  // edge axes u_i x v_j (codes 7 + 3 i + j)
  for (int i = 0; i < 3; ++i) {
    const int c1 = (i + 1) % 3, c2 = (i + 2) % 3;
    const int lo = i == 0 ? 1 : 0, hi = i == 2 ? 1 : 2;
    for (int j = 0; j < 3; ++j) {
      const int jlo = j == 0 ? 1 : 0, jhi = j == 2 ? 1 : 2;
      const double tmp = pp[c2] * R[c1][j] - pp[c1] * R[c2][j];
      const double s2 = std::abs(tmp) - (A[lo] * Q[hi][j] + A[hi] * Q[lo][j] + B[jlo] * Q[i][jhi] + B[jhi] * Q[i][jlo]);
      if (s2 > 0) { separation = s2; code = 0; return 0; }
      V3 n;
      n[i] = 0;
      n[c1] = -R[c2][j];
      n[c2] = R[c1][j];
      const double l = norm(n);
      if (l > eps) {
        const double s2n = s2 / l;
        if (s2n * fudge_factor > s) { s = s2n; best_col = -1; normalC = n / l; invert = tmp < 0; code = 7 + 3 * i + j; }
      }
    }
  }
  if (best_col != -1) normal = best_box == 1 ? col1(best_col) : col2(best_col);
  else normal = V3(dot(V3(r1(0, 0), r1(0, 1), r1(0, 2)), normalC), dot(V3(r1(1, 0), r1(1, 1), r1(1, 2)), normalC),
                   dot(V3(r1(2, 0), r1(2, 1), r1(2, 2)), normalC));
  if (invert) normal = -normal;
  depth = -s;
  if (code > 6) {
    // edge-edge: closest points of the two touching edges
    V3 pa = T1, pb = T2;
    for (int j = 0; j < 3; ++j) pa = pa + col1(j) * (A[j] * (dot(col1(j), normal) > 0 ? 1.0 : -1.0));
    for (int j = 0; j < 3; ++j) pb = pb + col2(j) * (B[j] * (dot(col2(j), normal) > 0 ? -1.0 : 1.0));
    const V3 ua = col1((code - 7) / 3), ub = col2((code - 7) % 3);
    double alpha, beta;
    lineClosestApproach(pa, ua, pb, ub, alpha, beta);
    pa = pa + ua * alpha;
    pb = pb + ub * beta;
    contacts[0] = BoxContact{normal, (pa + pb) * 0.5, depth};
    return 1;
  }
  // face-something: reference face on box a (codes 1-3: box 1), incident box b
  const bool ref1 = code <= 3;
  const double* Ra = ref1 ? R1 : R2;
  const double* Rb = ref1 ? R2 : R1;
  const V3 Pa = ref1 ? T1 : T2, Pb = ref1 ? T2 : T1;
  const V3 Sa = ref1 ? A : B, Sb = ref1 ? B : A;
  auto cola = [&](int c) { return V3(Ra[c], Ra[3 + c], Ra[6 + c]); };
  auto colb = [&](int c) { return V3(Rb[c], Rb[3 + c], Rb[6 + c]); };
  const V3 normal2 = ref1 ? normal : -normal;
  const V3 nr(dot(colb(0), normal2), dot(colb(1), normal2), dot(colb(2), normal2));
  const V3 anr(std::abs(nr[0]), std::abs(nr[1]), std::abs(nr[2]));
  int lanr, a1, a2;
  if (anr[1] > anr[0]) {
    if (anr[1] > anr[2]) { a1 = 0; lanr = 1; a2 = 2; }
    else { a1 = 0; a2 = 1; lanr = 2; }
  } else {
    if (anr[0] > anr[2]) { lanr = 0; a1 = 1; a2 = 2; }
    else { a1 = 0; a2 = 1; lanr = 2; }
  }
  const V3 center = nr[lanr] < 0 ? (Pb - Pa) + colb(lanr) * Sb[lanr] : (Pb - Pa) - colb(lanr) * Sb[lanr];
  const int codeN = ref1 ? code - 1 : code - 4;
  const int code1 = codeN == 0 ? 1 : 0, code2 = codeN == 2 ? 1 : 2;
  double quad[8];
  const double c1 = dot(cola(code1), center), c2 = dot(cola(code2), center);
  double m11 = dot(colb(a1), cola(code1)), m12 = dot(colb(a2), cola(code1));
  double m21 = dot(colb(a1), cola(code2)), m22 = dot(colb(a2), cola(code2));
  {
    const double k1 = m11 * Sb[a1], k2 = m21 * Sb[a1], k3 = m12 * Sb[a2], k4 = m22 * Sb[a2];
    quad[0] = c1 - k1 - k3;
    quad[1] = c2 - k2 - k4;
    quad[2] = c1 - k1 + k3;
    quad[3] = c2 - k2 + k4;
    quad[4] = c1 + k1 + k3;
    quad[5] = c2 + k2 + k4;
    quad[6] = c1 + k1 - k3;
    quad[7] = c2 + k2 - k4;
  }
  const double rect[2] = {Sa[code1], Sa[code2]};
  double ret[16];
  const int n_int = intersectRectQuad2(rect, quad, ret);
  if (n_int < 1) return 0;
  V3 points[8];
  double dep[8];
  const double det1 = (double)1.f / (m11 * m22 - m12 * m21);
  m11 *= det1;
  m12 *= det1;
  m21 *= det1;
  m22 *= det1;
  int cnum = 0;
  for (int j = 0; j < n_int; ++j) {
    const double k1 = m22 * (ret[j * 2] - c1) - m12 * (ret[j * 2 + 1] - c2);
    const double k2 = -m21 * (ret[j * 2] - c1) + m11 * (ret[j * 2 + 1] - c2);
    points[cnum] = center + colb(a1) * k1 + colb(a2) * k2;
    dep[cnum] = Sa[codeN] - dot(normal2, points[cnum]);
    if (dep[cnum] >= 0) {
      ret[cnum * 2] = ret[j * 2];
      ret[cnum * 2 + 1] = ret[j * 2 + 1];
      cnum++;
    }
  }
  if (cnum < 1) return 0;
  if (maxc > cnum) maxc = cnum;
  if (maxc < 1) maxc = 1;
  int iret[8] = {0, 1, 2, 3, 4, 5, 6, 7};
  if (cnum > maxc) {
    int i1 = 0;
    double maxdepth = dep[0];
    for (int i = 1; i < cnum; ++i)
      if (dep[i] > maxdepth) { maxdepth = dep[i]; i1 = i; }
    cullPoints2(cnum, ret, maxc, i1, iret);
    cnum = maxc;
  }
  for (int j = 0; j < cnum; ++j) {
    const int i = iret[j];
    const V3 half = normal * (dep[i] / 2);
    contacts[j] = BoxContact{normal, ref1 ? points[i] + Pa + half : points[i] + Pa - half, dep[i]};
  }
  return cnum;
}

// The solver fcl::collide picks for (a, b), with a at the origin and b posed
// by `pose`; false when the pair has no closed-form solver here.
inline bool analyticIntersect(const Shape& a, const Shape& b, const Iso& pose, AContact& out) {
  const bool sa = a.type == kSphere, sb = b.type == kSphere;
  if (a.type == kBox && b.type == kBox) {
    // boxBoxIntersect (box_box-inl.h:823-839): boxBox2 with at most 4 contacts;
    // the collision flag is its axis code.  A one-contact request keeps the
    // first contact of maximal depth (the partial sort by depth in
    // shape_pair_intersect-inl.h:92-104)
    const double I[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    BoxContact cts[4];
    V3 normal;
    double depth = 0, sep = 0;
    int code = 0;
    const int n = boxBox2(V3(a.p[0], a.p[1], a.p[2]), I, V3(0, 0, 0), V3(b.p[0], b.p[1], b.p[2]), pose.R, pose.t,
                          normal, depth, code, 4, cts, sep);
    out = AContact();
    out.hit = code != 0;
    if (!out.hit) {
      out.separation = sep;
    } else if (n > 0) {
      int k = 0;
      for (int j = 1; j < n; ++j)
        if (cts[j].depth > cts[k].depth) k = j;
      out.normal = cts[k].normal;
      out.pos = cts[k].pos;
      out.depth = cts[k].depth;
    } else {
      // a collision without a contact point (the clip came back empty)
      out.normal = normal;
      out.pos = pose.t * 0.5;
      out.depth = depth;
    }
    return true;
  }
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
