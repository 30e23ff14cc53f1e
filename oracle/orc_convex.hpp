// ORACLE — test infrastructure only.
//
// FP64 CPU restatement of mind-fcl's convex query engine (GJK boolean + GJK
// separation distance, EPA penetration, MPR boolean) and of the GJKSolver
// bridge that fcl::collide / GJKSolver::shapeSignedDistance run on top of it.
// It is the checker for the GPU kernels, never a product path: only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.
//
// Every function cites the reference file:line it restates (paths relative to
// the mind-fcl project root).  Arithmetic follows the operation order that the
// reference's Eigen expressions evaluate in (dot = (x0*y0 + x1*y1) + x2*y2,
// matrix*vector row by row, vector/scalar divides each coefficient), so that
// the restatement and the reference compiled through oracle/eigen_shim agree
// bit for bit when both are built with -ffp-contract=off.
//
// Convex support: the naive O(V) scan (include/fcl/geometry/shape/convex-inl.h:133-149)
// unless the shape carries a neighbour table (Convex::neighbors_ layout,
// convex-inl.h:379-405); then the reference's hill climb from six cached
// axis-extreme vertices (convex-inl.h:153-283), which fcl::Convex uses for
// hulls of more than 32 vertices.  Callers choose which shapes get a table.
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <limits>
#include <vector>

namespace orc {

// ---------------------------------------------------------------- vectors --
struct V3 {
  double x = 0, y = 0, z = 0;
  V3() = default;
  V3(double a, double b, double c) : x(a), y(b), z(c) {}
  double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
  double& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
};
inline V3 operator+(const V3& a, const V3& b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(const V3& a, const V3& b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator-(const V3& a) { return V3(-a.x, -a.y, -a.z); }
inline V3 operator*(const V3& a, double s) { return V3(a.x * s, a.y * s, a.z * s); }
inline V3 operator*(double s, const V3& a) { return V3(s * a.x, s * a.y, s * a.z); }
inline V3 operator/(const V3& a, double s) { return V3(a.x / s, a.y / s, a.z / s); }
inline double dot(const V3& a, const V3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline V3 cross(const V3& a, const V3& b) {
  return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline double sqn(const V3& a) { return dot(a, a); }
inline double norm(const V3& a) { return std::sqrt(sqn(a)); }
// Eigen's normalize(): leaves a zero vector unchanged.
inline void normalize(V3& a) {
  const double n2 = sqn(a);
  if (n2 > 0.0) {
    const double n = std::sqrt(n2);
    a = a / n;
  }
}
inline V3 normalized(V3 a) { normalize(a); return a; }
inline double absnorm(const V3& v) { return std::abs(v.x) + std::abs(v.y) + std::abs(v.z); }

// Row-major 3x3 rotation plus translation.
struct Iso {
  double R[9];
  V3 t;
  V3 rot(const V3& v) const {
    return V3((R[0] * v.x + R[1] * v.y) + R[2] * v.z, (R[3] * v.x + R[4] * v.y) + R[5] * v.z,
              (R[6] * v.x + R[7] * v.y) + R[8] * v.z);
  }
  V3 rotT(const V3& v) const {
    return V3((R[0] * v.x + R[3] * v.y) + R[6] * v.z, (R[1] * v.x + R[4] * v.y) + R[7] * v.z,
              (R[2] * v.x + R[5] * v.y) + R[8] * v.z);
  }
  V3 apply(const V3& v) const { return rot(v) + t; }
};

// ----------------------------------------------------------------- shapes --
// Shape type codes are GJKShapeType's values (include/fcl/cvx_collide/gjk_shape.h:9-28).
enum ShapeType : int32_t { kBox = 0, kSphere = 1, kCapsule = 3, kCylinder = 5, kConvex = 100, kTriangle = 101 };

struct Shape {
  int32_t type = kSphere;
  const float* verts = nullptr;  // xyzw, convex only
  int32_t nv = 0;
  double p[3] = {0, 0, 0};       // box: side; sphere: radius; capsule/cylinder: radius, lz
  V3 interior;                   // convex: vertex mean; primitives: zero
  const int32_t* nbr = nullptr;  // convex: neighbour table (walk), or null (scan)
  int start[6] = {0, 0, 0, 0, 0, 0};  // walk: extreme vertex along +x, -x, +y, -y, +z, -z
};

// Convex interior point = vertex mean, convex-inl.h:58-63.
inline V3 convexMean(const float* v, int n) {
  V3 sum;
  for (int i = 0; i < n; ++i) sum = sum + V3(v[4 * i], v[4 * i + 1], v[4 * i + 2]);
  return sum * (double)(1.0 / (double)n);
}

// Convex::findExtremeVertexIndexNaive, convex-inl.h:133-149 (first maximum).
inline int convexScan(const float* v, int n, const V3& d) {
  int best = 0;
  double best_val = dot(d, V3(v[0], v[1], v[2]));
  for (int i = 1; i < n; ++i) {
    const double val = dot(d, V3(v[4 * i], v[4 * i + 1], v[4 * i + 2]));
    if (val > best_val) { best = i; best_val = val; }
  }
  return best;
}

// Convex::initExtremeViaNeighborCache, convex-inl.h:153-199: the naive
// extreme vertex along each signed unit axis.
inline void initWalk(Shape& s, const int32_t* nbr) {
  s.nbr = nbr;
  const V3 axes[6] = {V3(1, 0, 0), V3(-1, 0, 0), V3(0, 1, 0), V3(0, -1, 0), V3(0, 0, 1), V3(0, 0, -1)};
  for (int k = 0; k < 6; ++k) s.start[k] = convexScan(s.verts, s.nv, axes[k]);
}

// Convex::findExtremeVertexViaNeighbours, convex-inl.h:201-283.
inline int convexWalk(const Shape& s, const V3& d) {
  const V3 axes[6] = {V3(1, 0, 0), V3(-1, 0, 0), V3(0, 1, 0), V3(0, -1, 0), V3(0, 0, 1), V3(0, 0, -1)};
  int init = -1;
  double max_dot = 0;
  for (int k = 0; k < 6; ++k) {
    const double dv = dot(axes[k], d);
    if (init < 0 || dv > max_dot) { init = s.start[k]; max_dot = dv; }
  }
  const float* v = s.verts;
  const int32_t* nb = s.nbr;
  int ext = init;
  double ext_val = dot(d, V3(v[4 * ext], v[4 * ext + 1], v[4 * ext + 2]));
  int parent0 = init, parent1 = init;
  bool keep = true;
  while (keep) {
    keep = false;
    const int first = nb[ext], count = nb[first], old = ext;
    for (int j = first + 1; j <= first + count; ++j) {
      const int n = nb[j];
      if (n == parent0 || n == parent1) continue;
      const double val = dot(d, V3(v[4 * n], v[4 * n + 1], v[4 * n + 2]));
      if (val > ext_val) {
        parent1 = ext;
        keep = true;
        ext = n;
        ext_val = val;
      }
    }
    parent0 = old;
  }
  return ext;
}

// Supports: gjk_shape.hpp:44-51 (box), :65-71 (sphere), :101-117 (capsule),
// :161-177 (cylinder); convex: Convex::findExtremeVertex, convex-inl.h:111-121.
inline V3 support(const Shape& s, const V3& d) {
  switch (s.type) {
    case kBox:
      return V3((d[0] > 0) ? (s.p[0] / 2) : (-s.p[0] / 2), (d[1] > 0) ? (s.p[1] / 2) : (-s.p[1] / 2),
                (d[2] > 0) ? (s.p[2] / 2) : (-s.p[2] / 2));
    case kSphere:
      return d * s.p[0];
    case kCapsule: {
      const double r = s.p[0], half_h = s.p[1] * 0.5;
      V3 pos1(0, 0, half_h), pos2(0, 0, -half_h);
      const V3 v = d * r;
      pos1 = pos1 + v;
      pos2 = pos2 + v;
      return (dot(d, pos1) > dot(d, pos2)) ? pos1 : pos2;
    }
    case kCylinder: {
      const double r = s.p[0];
      const double zdist = std::sqrt(d[0] * d[0] + d[1] * d[1]);
      const double half_h = s.p[1] * 0.5;
      if (zdist == 0.0) return V3(0, 0, (d[2] > 0) ? half_h : -half_h);
      const double k = r / zdist;
      return V3(k * d[0], k * d[1], (d[2] > 0) ? half_h : -half_h);
    }
    case kConvex: {
      const float* v = s.verts;
      const int best = s.nbr ? convexWalk(s, d) : convexScan(v, s.nv, d);
      return V3(v[4 * best], v[4 * best + 1], v[4 * best + 2]);
    }
    case kTriangle: {
      // triangleSupport, geometry/shape/shape_gjk_interface-inl.h:17-39
      const float* v = s.verts;
      const V3 a(v[0], v[1], v[2]), b(v[4], v[5], v[6]), c(v[8], v[9], v[10]);
      const double da = dot(d, a), db = dot(d, b), dc = dot(d, c);
      if (da > db) return dc > da ? c : a;
      return dc > db ? c : b;
    }
    default:
      return V3();
  }
}

// ---------------------------------------------------- Minkowski difference --
// minkowski_diff.hpp:21-85.  toshape0 = pose of shape 1 in shape 0's frame,
// toshape1 = its rotation transposed (gjk_solver-inl.h:84-85).
struct MinkVertex {
  V3 vertex, direction;
};
struct MinkDiff {
  const Shape* s0;
  const Shape* s1;
  Iso to0;
  // Shape 0 swept along `sweep` (its frame) when `swept`: the ShapeSweptVolume
  // support and interior of computeSupport / computeInterior
  // (narrowphase/detail/gjk_solver_cvx-inl.h:90-107, 128-141).
  bool swept = false;
  V3 sweep;
  V3 support0(const V3& d) const {
    const V3 p = orc::support(*s0, d);
    return (swept && dot(d, sweep) > 0) ? p + sweep : p;
  }
  V3 support1(const V3& d) const { return to0.apply(orc::support(*s1, to0.rotT(d))); }
  V3 support(const V3& d) const { return support0(d) - support1(-d); }
  MinkVertex supportVertex(const V3& d) const {
    MinkVertex v;
    v.direction = d;
    v.vertex = support0(d) - support1(-d);
    return v;
  }
  V3 interior() const {
    const V3 i0 = swept ? s0->interior + sweep * 0.5 : s0->interior;
    return i0 - to0.apply(s1->interior);
  }
};

// -------------------------------------------------------------------- GJK --
enum class GJKStatus : int { Intersect = 0, Separated = 1, ConvergeNoProgress = 2, IterationLimit = 3, Failed = 4 };

struct Simplex {
  MinkVertex v[4];
  int rank = -1;
  void reset() { rank = -1; }
  bool valid() const { return rank > 0; }
  void add(const MinkVertex& x) {
    if (rank < 0) rank = 0;
    v[rank] = x;
    rank += 1;
  }
};

struct MinDistOut {
  bool certify_valid = false;
  MinkVertex certify;
  bool point_valid = false;
  V3 p0, p1;
};

class GJK {
 public:
  GJK(int max_iter, double tol) : max_iter_(max_iter), tol_(tol) {}
  int iterations = 0;  // support-loop iterations of the last Evaluate (boolean + distance)

  // gjk.hpp:10-140
  GJKStatus Evaluate(const MinkDiff& shape, Simplex& simplex, const V3& guess, MinDistOut* out) {
    iterations = 0;
    V3 direction = guess;
    if (sqn(direction) <= 0.0) direction = V3(1, 0, 0);
    normalize(direction);

    MinkVertex vertex = shape.supportVertex(direction);
    simplex.reset();
    simplex.add(vertex);
    const double tol2 = tol_ * tol_;
    if (sqn(vertex.vertex) <= tol2) return GJKStatus::Intersect;
    if (dot(vertex.vertex, direction) < 0) return separated(shape, simplex, vertex, out);

    direction = -direction;
    int iteration = 0;
    while (iteration < max_iter_) {
      iteration += 1;
      iterations = iteration;
      vertex = shape.supportVertex(direction);
      if (dot(vertex.vertex, direction) < 0) return separated(shape, simplex, vertex, out);
      for (int j = 0; j < simplex.rank; ++j) {
        if (sqn(simplex.v[j].vertex - vertex.vertex) < tol2)
          return undetermined(shape, simplex, GJKStatus::ConvergeNoProgress, out);
      }
      if (sqn(vertex.vertex) <= tol2) {
        simplex.add(vertex);
        return GJKStatus::Intersect;
      }
      simplex.add(vertex);
      Proj st = project(simplex, direction);
      if (st == Proj::Failed) return GJKStatus::Failed;
      if (st == Proj::Intersect) return GJKStatus::Intersect;
      if (st == Proj::ZeroVolume) return undetermined(shape, simplex, GJKStatus::ConvergeNoProgress, out);
    }
    return undetermined(shape, simplex, GJKStatus::IterationLimit, out);
  }

 private:
  int max_iter_;
  double tol_;
  static constexpr double kBaryTol = 1e-3;  // gjk.h:131
  enum class Proj { Failed, Continue, Intersect, ZeroVolume };
  enum class Upd { NoImprovement, OK, Failed };

  // gjk.hpp:22-51
  GJKStatus separated(const MinkDiff& shape, Simplex& simplex, const MinkVertex& sv, MinDistOut* out) {
    if (out == nullptr) return GJKStatus::Separated;
    out->certify_valid = true;
    out->certify = sv;
    simplex.reset();
    simplex.add(sv);
    V3 p0, p1;
    const bool ok = minDistanceFromSeparated(shape, simplex, p0, p1);
    out->point_valid = ok;
    if (ok) { out->p0 = p0; out->p1 = p1; }
    return GJKStatus::Separated;
  }
  // gjk.hpp:53-73
  GJKStatus undetermined(const MinkDiff& shape, Simplex& simplex, GJKStatus st, MinDistOut* out) {
    if (out != nullptr) {
      out->certify_valid = false;
      V3 p0, p1;
      const bool ok = extractTrySub(shape, simplex, p0, p1);
      out->point_valid = ok;
      if (ok) { out->p0 = p0; out->p1 = p1; }
    }
    return st;
  }

  // gjk.hpp:142-159
  Proj project(Simplex& s, V3& d) const {
    if (s.rank == 2) return project2(s, d);
    if (s.rank == 3) return project3(s, d);
    return project4(s, d);
  }
  // gjk.hpp:161-197
  Proj project2(Simplex& s, V3& d) const {
    const MinkVertex B = s.v[0], A = s.v[1];
    const V3& a = A.vertex;
    const V3& b = B.vertex;
    const V3 a_to_b = b - a;
    const double ao_dot_ab = -dot(a_to_b, a);
    const V3 ab_cross_ao = cross(a, a_to_b);
    if (ao_dot_ab > 0 && sqn(ab_cross_ao) <= 0.0) return Proj::Intersect;
    if (ao_dot_ab <= 0) {
      s.reset();
      s.add(A);
      d = -normalized(a);
      return Proj::Continue;
    }
    d = cross(ab_cross_ao, a_to_b);
    normalize(d);
    return Proj::Continue;
  }
  // gjk.hpp:199-278
  Proj project3(Simplex& s, V3& d) const {
    const MinkVertex C = s.v[0], B = s.v[1], A = s.v[2];
    const V3& a = A.vertex;
    const V3& b = B.vertex;
    const V3& c = C.vertex;
    const V3 a_to_b = b - a;
    const V3 a_to_c = c - a;
    const bool a_sep_b = dot(a, a_to_b) >= 0;
    const bool a_sep_c = dot(a, a_to_c) >= 0;
    if (a_sep_b && a_sep_c) {
      s.reset();
      s.add(A);
      d = -a;
      normalize(d);
      return Proj::Continue;
    }
    const V3 n = cross(a_to_b, a_to_c);
    const V3 ac_normal = cross(n, a_to_c);
    if (dot(a, ac_normal) <= 0) {
      s.v[1] = A;
      s.rank = 2;
      const V3 ac_cross_ao = cross(a, a_to_c);
      d = cross(ac_cross_ao, a_to_c);
      normalize(d);
      return Proj::Continue;
    }
    const V3 ab_normal = cross(a_to_b, n);
    if (dot(a, ab_normal) <= 0) {
      s.v[0] = B;
      s.v[1] = A;
      s.rank = 2;
      const V3 ab_cross_ao = cross(a, a_to_b);
      d = cross(ab_cross_ao, a_to_b);
      normalize(d);
      return Proj::Continue;
    }
    const double area = norm(n);
    if (area < tol_ * tol_) return Proj::Failed;
    const V3 nu = n / area;
    const double nu_dot_a = dot(nu, a);
    if (std::abs(nu_dot_a) < tol_) return Proj::Intersect;
    d = (nu_dot_a <= 0) ? nu : -nu;
    return Proj::Continue;
  }
  // gjk.hpp:280-360
  Proj project4(Simplex& s, V3& dir) const {
    const MinkVertex D = s.v[0], C = s.v[1], B = s.v[2], A = s.v[3];
    const V3& a = A.vertex;
    const V3& b = B.vertex;
    const V3& c = C.vertex;
    const V3& d = D.vertex;
    const V3 ab = b - a, ac = c - a, ad = d - a;
    V3 abc = cross(ab, ac), acd = cross(ac, ad), abd = cross(ab, ad);
    double abc_ad = dot(abc, ad), acd_ab = dot(acd, ab), abd_ac = dot(abd, ac);
    if (std::abs(abc_ad) <= 0.0) return Proj::ZeroVolume;
    if (abc_ad > 0) { abc = -abc; abc_ad = -abc_ad; }
    if (acd_ab > 0) { acd = -acd; acd_ab = -acd_ab; }
    if (abd_ac > 0) { abd = -abd; abd_ac = -abd_ac; }
    const bool d_side = dot(a, abc) > 0;
    const bool c_side = dot(a, abd) > 0;
    const bool b_side = dot(a, acd) > 0;
    if (d_side && c_side && b_side) return Proj::Intersect;
    if (!b_side) {
      s.v[2] = A;
      s.rank = 3;
    } else if (!c_side) {
      s.v[1] = B;
      s.v[2] = A;
      s.rank = 3;
    } else {
      s.v[0] = C;
      s.v[1] = B;
      s.v[2] = A;
      s.rank = 3;
    }
    return project3(s, dir);
  }

  // gjk_distance.hpp:10-105
  bool minDistanceFromSeparated(const MinkDiff& shape, Simplex& s, V3& p0, V3& p1) {
    if (s.rank != 1) return false;
    V3 cur;
    if (updateSimplex(s, cur) != Upd::OK) return false;
    double book = norm(cur);
    if (book <= tol_) return extractNoSub(shape, s, p0, p1);
    V3 next = -cur / book;
    const double tol2 = tol_ * tol_;
    int iteration = 0;
    while (iteration < max_iter_) {
      iteration += 1;
      iterations += 1;
      const MinkVertex nv = shape.supportVertex(next);
      if (dot(next, nv.vertex - cur) < tol_) return extractNoSub(shape, s, p0, p1);
      for (int j = 0; j < s.rank; ++j)
        if (sqn(s.v[j].vertex - nv.vertex) < tol2) return extractNoSub(shape, s, p0, p1);
      s.add(nv);
      const Upd st = updateSimplex(s, cur);
      if (st == Upd::NoImprovement) return extractNoSub(shape, s, p0, p1);
      if (st != Upd::OK) return false;
      const double nd = norm(cur);
      if (book - nd < tol_) return extractNoSub(shape, s, p0, p1);
      if (nd < tol_) return extractNoSub(shape, s, p0, p1);
      book = nd;
      next = -cur / book;
    }
    return false;
  }
  // gjk_distance.hpp:107-126
  Upd updateSimplex(Simplex& s, V3& out) const {
    if (s.rank == 1) { out = s.v[0].vertex; return Upd::OK; }
    if (s.rank == 2) { update2(s, out); return Upd::OK; }
    if (s.rank == 3) { update3(s, out); return Upd::OK; }
    if (s.rank == 4) return update4(s, out);
    return Upd::Failed;
  }
  // gjk_distance.hpp:128-153
  void update2(Simplex& s, V3& out) const {
    const V3 s1 = s.v[1].vertex;
    const V3 s2 = s.v[0].vertex;
    const V3 s1_to_s2 = s2 - s1;
    const double len2 = sqn(s1_to_s2);
    const double t = -dot(s1, s1_to_s2);
    if (t <= 0 || len2 <= tol_ * tol_) {
      out = s1;
      s.v[0] = s.v[1];
      s.rank = 1;
    } else if (t >= len2) {
      out = s2;
      s.rank = 1;
    } else {
      const double w2 = t / len2;
      out = w2 * s2 + (1.0 - w2) * s1;
    }
  }
  // gjk_distance.hpp:155-286
  void update3(Simplex& s, V3& out) const {
    const V3 s1 = s.v[2].vertex;
    const V3 s2 = s.v[1].vertex;
    const V3 s3 = s.v[0].vertex;
    const V3 s1_to_s2 = s2 - s1;
    const V3 s1_to_s3 = s3 - s1;
    const bool sep_s2 = dot(s1, s1_to_s2) >= 0;
    const bool sep_s3 = dot(s1, s1_to_s3) >= 0;
    if (sep_s2 && sep_s3) {
      out = s1;
      s.v[0] = s.v[2];
      s.rank = 1;
      return;
    }
    const V3 n = cross(s1_to_s2, s1_to_s3);
    const double area2 = sqn(n);
    const bool zero_area = area2 <= 0.0;
    const V3 n12 = cross(n, s1_to_s2);
    const bool s12_sep = dot(s1, n12) > 0;
    if (!sep_s2 && s12_sep) {
      s.v[0] = s.v[1];
      s.v[1] = s.v[2];
      s.rank = 2;
      update2(s, out);
      return;
    }
    const V3 n13 = cross(n, s1_to_s3);
    const bool s13_sep = dot(s1, n13) < 0;
    if (!sep_s3 && s13_sep) {
      s.v[1] = s.v[2];
      s.rank = 2;
      update2(s, out);
      return;
    }
    double best = -1;
    V3 best_pt, cache_pt;
    Simplex best_s, cache;
    if (zero_area || s12_sep) {
      cache = s;
      cache.v[0] = cache.v[1];
      cache.v[1] = cache.v[2];
      cache.rank = 2;
      update2(cache, cache_pt);
      const double dd = sqn(cache_pt);
      if (best < 0 || dd < best) { best = dd; best_s = cache; best_pt = cache_pt; }
    }
    if (zero_area || s13_sep) {
      cache = s;
      cache.v[1] = cache.v[2];
      cache.rank = 2;
      update2(cache, cache_pt);
      const double dd = sqn(cache_pt);
      if (best < 0 || dd < best) { best = dd; best_s = cache; best_pt = cache_pt; }
    }
    const V3 n23 = cross(n, s3 - s2);
    const bool s23_sep = dot(s2, n23) > 0;
    if (zero_area || s23_sep) {
      cache = s;
      cache.rank = 2;
      update2(cache, cache_pt);
      const double dd = sqn(cache_pt);
      if (best < 0 || dd < best) { best = dd; best_s = cache; best_pt = cache_pt; }
    }
    if (best < 0) {
      const double d = dot(s1, n);
      out = n * (d / area2);
    } else {
      s = best_s;
      out = best_pt;
    }
  }
  // gjk_distance.hpp:288-373
  Upd update4(Simplex& s, V3& out) const {
    double best = -1;
    V3 best_pt, cache_pt;
    Simplex best_s, cache;
    // faces (3,2,1), (3,2,0), (3,1,0) in the order the reference tries them
    cache = s;
    cache.v[0] = cache.v[1];
    cache.v[1] = cache.v[2];
    cache.v[2] = cache.v[3];
    cache.rank = 3;
    update3(cache, cache_pt);
    double dd = sqn(cache_pt);
    if (best < 0 || dd < best) { best = dd; best_pt = cache_pt; best_s = cache; }
    cache = s;
    cache.v[1] = cache.v[2];
    cache.v[2] = cache.v[3];
    cache.rank = 3;
    update3(cache, cache_pt);
    dd = sqn(cache_pt);
    if (best < 0 || dd < best) { best = dd; best_pt = cache_pt; best_s = cache; }
    cache = s;
    cache.v[2] = cache.v[3];
    cache.rank = 3;
    update3(cache, cache_pt);
    dd = sqn(cache_pt);
    if (best < 0 || dd < best) { best = dd; best_pt = cache_pt; best_s = cache; }
    if (best < 0) return Upd::NoImprovement;
    s = best_s;
    out = best_pt;
    return Upd::OK;
  }
  // gjk_distance.hpp:375-470
  bool extractNoSub(const MinkDiff& shape, const Simplex& s, V3& p0, V3& p1) const {
    if (s.rank == 4 || !s.valid()) return false;
    if (s.rank == 1) {
      p0 = shape.support0(s.v[0].direction);
      p1 = shape.support1(-s.v[0].direction);
      return true;
    }
    if (s.rank == 2) {
      const MinkVertex& v1 = s.v[0];
      const MinkVertex& v2 = s.v[1];
      const V3 s1_to_s2 = v2.vertex - v1.vertex;
      const double len2 = sqn(s1_to_s2);
      if (len2 <= 0.0) {
        p0 = shape.support0(v1.direction);
        p1 = shape.support1(-v1.direction);
        return true;
      }
      const double t = -dot(v1.vertex, s1_to_s2);
      const double w2 = t / len2;
      if (w2 > 1 + kBaryTol) {
        p0 = shape.support0(v2.direction);
        p1 = shape.support1(-v2.direction);
        return false;
      } else if (w2 < -kBaryTol) {
        p0 = shape.support0(v1.direction);
        p1 = shape.support1(-v1.direction);
        return false;
      }
      const double w1 = 1.0 - w2;
      p0 = shape.support0(v1.direction) * w1 + shape.support0(v2.direction) * w2;
      p1 = shape.support1(-v1.direction) * w1 + shape.support1(-v2.direction) * w2;
      return true;
    }
    const MinkVertex& v1 = s.v[0];
    const MinkVertex& v2 = s.v[1];
    const MinkVertex& v3 = s.v[2];
    const V3 s1_to_s2 = v2.vertex - v1.vertex;
    const V3 s1_to_s3 = v3.vertex - v1.vertex;
    const V3 n = cross(s1_to_s2, s1_to_s3);
    const double area2 = sqn(n);
    if (area2 <= 0.0) return false;
    const double d = dot(v1.vertex, n);
    const V3 proj = n * (d / area2);
    const double area = std::sqrt(area2);
    const double w2 = norm(cross(s1_to_s3, v1.vertex - proj)) / area;
    const double w3 = norm(cross(s1_to_s2, v1.vertex - proj)) / area;
    const double w1 = 1.0 - w2 - w3;
    if (w1 < -kBaryTol || w2 < -kBaryTol || w3 < -kBaryTol) return false;
    p0 = (shape.support0(v1.direction) * w1 + shape.support0(v2.direction) * w2) + shape.support0(v3.direction) * w3;
    p1 = (shape.support1(-v1.direction) * w1 + shape.support1(-v2.direction) * w2) + shape.support1(-v3.direction) * w3;
    return true;
  }
  // gjk_distance.hpp:472-559
  bool extractTrySub(const MinkDiff& shape, const Simplex& s, V3& p0, V3& p1) const {
    if (s.rank >= 4) return false;
    if (s.rank <= 2) {
      extractNoSub(shape, s, p0, p1);
      return true;
    }
    double best = -1;
    V3 b0, b1, c0, c1;
    Simplex cache = s;
    if (extractNoSub(shape, cache, c0, c1)) {
      const double dd = sqn(c0 - c1);
      if (best < 0 || dd < best) { best = dd; b0 = c0; b1 = c1; }
    }
    cache = s;
    cache.rank = 2;
    extractNoSub(shape, cache, c0, c1);
    double dd = sqn(c0 - c1);
    if (best < 0 || dd < best) { best = dd; b0 = c0; b1 = c1; }
    cache = s;
    cache.v[1] = cache.v[2];
    cache.rank = 2;
    extractNoSub(shape, cache, c0, c1);
    dd = sqn(c0 - c1);
    if (best < 0 || dd < best) { best = dd; b0 = c0; b1 = c1; }
    cache = s;
    cache.v[0] = cache.v[1];
    cache.v[1] = cache.v[2];
    cache.rank = 2;
    extractNoSub(shape, cache, c0, c1);
    dd = sqn(c0 - c1);
    if (best < 0 || dd < best) { best = dd; b0 = c0; b1 = c1; }
    p0 = b0;
    p1 = b1;
    return true;
  }
};

// ----------------------------------------------------- polytope geometry --
struct MinDist {
  bool in = false;
  double sq = 0;
  V3 w;
};

// epa_polytope_utils.h:19-48.  For p != origin the in-segment branch keeps the
// reference's behaviour of returning |witness|^2 (not |witness - p|^2).
inline void pointToSegment(const V3& p, const V3& x0, const V3& x1, bool& in, double& sq, V3* w) {
  const V3 d = x1 - x0;
  const V3 a = x0 - p;
  const double dl2 = sqn(d);
  const double t = -1.0 * dot(a, d) / dl2;
  if (t <= 0.0) {
    if (w) *w = x0;
    in = false;
    sq = sqn(x0 - p);
  } else if (t >= 1.0) {
    if (w) *w = x1;
    in = false;
    sq = sqn(x1 - p);
  } else {
    const V3 lw = x0 + t * d;
    if (w) *w = lw;
    in = true;
    sq = sqn(lw);
  }
}
inline void pointToSegment(const V3& p, const V3& x0, const V3& x1, MinDist& m) { pointToSegment(p, x0, x1, m.in, m.sq, &m.w); }

// epa_polytope_utils.h:58-69
inline double pointToLine(const V3& p, const V3& a, const V3& b) {
  const V3 ab = b - a;
  const double len = norm(ab);
  if (len <= 0.0) return norm(p - a);
  return norm(cross(p - a, ab)) / len;
}
// epa_polytope_utils.h:71-86
inline double pointToPlane(const V3& p, const V3& a, const V3& b, const V3& c) {
  const V3 n = cross(a - b, b - c);
  const double nl = norm(n);
  if (nl <= 0.0) return pointToLine(p, a, b);
  const V3 un = n / nl;
  return std::abs(dot(un, a - p));
}
// epa_polytope_utils.h:88-165
inline void pointToTriangle(const V3& p, const V3& a, const V3& b, const V3& c, MinDist& m) {
  const V3 dl0 = a - b, dl1 = b - c, dl2 = c - a;
  const V3 n = cross(dl0, dl1);
  const double n2 = sqn(n);
  const double area = std::sqrt(n2);
  auto sub = [&]() {
    MinDist e[3];
    pointToSegment(p, a, b, e[0]);
    pointToSegment(p, b, c, e[1]);
    pointToSegment(p, c, a, e[2]);
    int k = 0;
    for (int i = 1; i < 3; ++i)
      if (e[i].sq < e[k].sq) k = i;
    m.in = false;
    m.sq = e[k].sq;
    m.w = e[k].w;
  };
  if (std::abs(area) <= 1e-16) { sub(); return; }
  const double d = dot(a - p, n);
  const V3 p2proj = n * (d / n2);
  const V3 proj = p + p2proj;
  double w[3];
  w[0] = norm(cross(dl1, b - proj)) / area;
  w[1] = norm(cross(dl2, c - proj)) / area;
  w[2] = 1.0 - w[0] - w[1];
  bool in = true;
  for (int i = 0; i < 3; ++i)
    if (w[i] < 0.0 || w[i] > 1.0) { in = false; break; }
  const double chk = norm(cross(dl0, a - proj)) / area;
  if (std::abs(chk - w[2]) > 1e-3) in = false;
  if (in) {
    m.in = true;
    m.sq = sqn(p2proj);
    m.w = (a * w[0] + b * w[1]) + c * w[2];
    return;
  }
  sub();
}

// --------------------------------------------------------------- polytope --
// epa_polytope.h / epa_polytope.hpp / epa_polytope_expand.hpp.  The reference
// keeps vertices/edges/faces in intrusive singly linked lists that new
// elements are prepended to, so every list is visited newest first; here the
// elements live in append-only arrays visited from the back, which is the same
// order.  Capacities count live elements as the reference's free lists do.
enum class FeatType { None, Vertex, Edge, Face };
enum class EdgeVis { Unknown, Border, Internal };
enum class FaceVis { Unknown, Visible, Hidden };

class Polytope {
 public:
  struct PV { V3 loc, dir; MinDist md; bool remove = false; int to_new = -1; bool alive = true; };
  struct PE { int v[2]; int f[2]; MinDist md; EdgeVis vis = EdgeVis::Unknown; bool alive = true; };
  struct PF { int e[3]; MinDist md; FaceVis vis = FaceVis::Unknown; bool alive = true; };
  std::vector<PV> V;
  std::vector<PE> E;
  std::vector<PF> F;

  explicit Polytope(size_t max_faces) { reset(max_faces); }
  // epa_polytope.hpp:80-103
  void reset(size_t max_faces) {
    cap_f_ = max_faces;
    cap_e_ = (size_t)(1.51 * (double)max_faces);
    cap_v_ = (size_t)(1.51 * (double)max_faces);
    V.clear(); E.clear(); F.clear();
    live_v_ = live_e_ = live_f_ = 0;
  }
  size_t face_capacity() const { return cap_f_; }

  // epa_polytope.hpp:160-186
  int addVertex(const MinkVertex& mv) {
    if (live_v_ >= cap_v_) return -1;
    PV v;
    v.loc = mv.vertex;
    v.dir = mv.direction;
    v.md.in = true;
    v.md.w = mv.vertex;
    v.md.sq = sqn(mv.vertex);
    V.push_back(v);
    live_v_++;
    return (int)V.size() - 1;
  }
  // epa_polytope.hpp:188-214
  int addEdge(int v1, int v2) {
    if (v1 < 0 || v2 < 0) return -1;
    if (live_e_ >= cap_e_) return -1;
    PE e;
    e.v[0] = v1;
    e.v[1] = v2;
    e.f[0] = e.f[1] = -1;
    pointToSegment(V3(), V[v1].loc, V[v2].loc, e.md);
    E.push_back(e);
    live_e_++;
    return (int)E.size() - 1;
  }
  // epa_polytope.hpp:216-265; -1 also when an edge already has two faces.
  int addFace(int e1, int e2, int e3) {
    if (e1 < 0 || e2 < 0 || e3 < 0) return -1;
    if (live_f_ >= cap_f_) return -1;
    PF f;
    f.e[0] = e1; f.e[1] = e2; f.e[2] = e3;
    const V3 a = V[E[e1].v[0]].loc;
    const V3 b = V[E[e1].v[1]].loc;
    const PE& eb = E[e2];
    const int cv = (eb.v[0] != E[e1].v[0] && eb.v[0] != E[e1].v[1]) ? eb.v[0] : eb.v[1];
    pointToTriangle(V3(), a, b, V[cv].loc, f.md);
    F.push_back(f);
    live_f_++;
    const int fi = (int)F.size() - 1;
    for (int i = 0; i < 3; ++i) {
      PE& ei = E[F[fi].e[i]];
      if (ei.f[0] < 0) {
        ei.f[0] = fi;
      } else {
        if (ei.f[1] >= 0) return -1;
        ei.f[1] = fi;
      }
    }
    return fi;
  }
  // epa_polytope.hpp:12-37
  void faceVerts(int fi, int& a, int& b, int& c) const {
    const PE& e0 = E[F[fi].e[0]];
    a = e0.v[0];
    b = e0.v[1];
    const PE& e1 = E[F[fi].e[1]];
    c = (e1.v[0] != a && e1.v[0] != b) ? e1.v[0] : e1.v[1];
  }

  // epa_polytope.hpp:267-345
  FeatType nearest(bool exclude_vertex, int& idx) const {
    idx = -1;
    if (live_v_ == 0) return FeatType::None;
    double best = std::numeric_limits<double>::infinity();
    FeatType bt = FeatType::None;
    if (!exclude_vertex) {
      for (int i = (int)V.size() - 1; i >= 0; --i) {
        if (!V[i].alive) continue;
        if (V[i].md.sq < best) { best = V[i].md.sq; bt = FeatType::Vertex; idx = i; }
      }
    }
    for (int i = (int)E.size() - 1; i >= 0; --i) {
      if (!E[i].alive) continue;
      if (!exclude_vertex && !E[i].md.in) continue;
      if (E[i].md.sq < best) { best = E[i].md.sq; bt = FeatType::Edge; idx = i; }
    }
    for (int i = (int)F.size() - 1; i >= 0; --i) {
      if (!F[i].alive) continue;
      if (!F[i].md.in) continue;
      if (F[i].md.sq < best) { best = F[i].md.sq; bt = FeatType::Face; idx = i; }
    }
    return bt;
  }

  // epa_polytope.hpp:347-411
  bool faceNormalOut(int fi, V3& n, double* area) const {
    int ia, ib, ic;
    faceVerts(fi, ia, ib, ic);
    const V3 a = V[ia].loc, b = V[ib].loc, c = V[ic].loc;
    const V3 e1 = a - b, e2 = b - c;
    const V3 cr = cross(e1, e2);
    const double nl = norm(cr);
    if (area) *area = 0.5 * nl;
    if (nl <= 0.0) return false;
    const V3 od = cr / nl;
    const double oa = dot(a, od);
    if (std::abs(oa) >= 1e-4) {
      n = (oa > 0) ? od : -od;
      return true;
    }
    double maxp = 0.0, minn = 0.0;
    for (int i = (int)V.size() - 1; i >= 0; --i) {
      if (!V[i].alive) continue;
      const double dv = dot(V[i].loc, od);
      if (dv > maxp) maxp = dv;
      if (dv < minn) minn = dv;
    }
    n = (std::abs(maxp) > std::abs(minn)) ? -od : od;
    return true;
  }
  // epa_polytope_expand.hpp:12-29
  bool pointOutside(int fi, const V3& p) const {
    V3 n;
    double area = 0;
    if (!faceNormalOut(fi, n, &area)) return area <= 0.0;
    const V3& onf = V[E[F[fi].e[0]].v[0]].loc;
    return dot(n, p - onf) >= 0.0;
  }

  enum class Expand { OK, Failed, MallocFailed };
  // epa_polytope_expand.hpp:31-86
  Expand expand(const MinkVertex& nv, int start_face) {
    for (auto& v : V) if (v.alive) { v.remove = true; v.to_new = -1; }
    for (auto& e : E) if (e.alive) e.vis = EdgeVis::Unknown;
    for (auto& f : F) if (f.alive) f.vis = FaceVis::Unknown;
    if (!visiblePatch(start_face, nv.vertex)) return Expand::Failed;
    // updateVertexRemoveFlag, epa_polytope_expand.hpp:183-206
    for (auto& e : E) {
      if (!e.alive) continue;
      if (e.vis != EdgeVis::Internal) { V[e.v[0]].remove = false; V[e.v[1]].remove = false; }
    }
    // removeAccordingToVisibility, epa_polytope_expand.hpp:242-279
    for (int i = (int)F.size() - 1; i >= 0; --i) {
      PF& f = F[i];
      if (!f.alive || f.vis != FaceVis::Visible) continue;
      for (int k = 0; k < 3; ++k) {
        PE& ek = E[f.e[k]];
        if (ek.f[0] == i) ek.f[0] = ek.f[1];
        ek.f[1] = -1;
      }
      f.alive = false;
      live_f_--;
    }
    for (auto& e : E) if (e.alive && e.vis == EdgeVis::Internal) { e.alive = false; live_e_--; }
    for (auto& v : V) if (v.alive && v.remove) { v.alive = false; live_v_--; }
    const int nvi = addVertex(nv);
    if (nvi < 0) return Expand::MallocFailed;
    const int n_edges_before = (int)E.size();
    for (int i = n_edges_before - 1; i >= 0; --i) {
      if (!E[i].alive || E[i].vis != EdgeVis::Border) continue;
      int ee[2];
      for (int k = 0; k < 2; ++k) {
        const int vk = E[i].v[k];
        if (V[vk].to_new < 0) V[vk].to_new = addEdge(nvi, vk);
        ee[k] = V[vk].to_new;
      }
      if (addFace(i, ee[0], ee[1]) < 0) return Expand::MallocFailed;
    }
    return Expand::OK;
  }

 private:
  size_t cap_f_ = 0, cap_e_ = 0, cap_v_ = 0;
  size_t live_v_ = 0, live_e_ = 0, live_f_ = 0;

  // epa_polytope_expand.hpp:120-180
  bool visiblePatch(int start, const V3& p) {
    struct Task { int f, k; };
    std::vector<Task> st;
    F[start].vis = FaceVis::Visible;
    for (int k = 0; k < 3; ++k) st.push_back({start, k});
    while (!st.empty()) {
      const Task t = st.back();
      st.pop_back();
      const int ei = F[t.f].e[t.k];
      if (ei < 0) return false;
      PE& e = E[ei];
      const int g = (e.f[0] == t.f) ? e.f[1] : e.f[0];
      if (g < 0) return false;
      if (F[g].vis == FaceVis::Visible) { e.vis = EdgeVis::Internal; continue; }
      if (F[g].vis == FaceVis::Hidden) { e.vis = EdgeVis::Border; continue; }
      if (pointOutside(g, p)) {
        F[g].vis = FaceVis::Visible;
        e.vis = EdgeVis::Internal;
        for (int k = 0; k < 3; ++k) st.push_back({g, k});
      } else {
        F[g].vis = FaceVis::Hidden;
        e.vis = EdgeVis::Border;
      }
    }
    return true;
  }
};

// -------------------------------------------------------------------- EPA --
enum class EPAStatus : int { Failed = 0, OK = 1, Touching = 2, IterationLimit = 3, MallocFailed = 4 };
enum class S2P { OK, Touching, Failed };

// epa_simplex2polytope.hpp:10-39
inline void touchingPoint(const MinkDiff& shape, const V3& d, V3& p0, V3& p1) {
  const V3 mid = (shape.support0(d) + shape.support1(-d)) / 2;
  p0 = mid;
  p1 = mid;
}

// epa_simplex2polytope.hpp:143-174
inline S2P formTetra(const MinkVertex& a, const MinkVertex& b, const MinkVertex& c, const MinkVertex& d, Polytope& P) {
  P.reset(P.face_capacity());
  int v[4] = {P.addVertex(a), P.addVertex(b), P.addVertex(c), P.addVertex(d)};
  int e[6] = {P.addEdge(v[0], v[1]), P.addEdge(v[1], v[2]), P.addEdge(v[2], v[0]),
              P.addEdge(v[3], v[0]), P.addEdge(v[3], v[1]), P.addEdge(v[3], v[2])};
  int f[4];
  f[0] = P.addFace(e[0], e[1], e[2]);
  f[1] = P.addFace(e[3], e[4], e[0]);
  f[2] = P.addFace(e[4], e[5], e[1]);
  f[3] = P.addFace(e[5], e[3], e[2]);
  for (int i = 0; i < 4; ++i) if (f[i] < 0) return S2P::Failed;
  return S2P::OK;
}

// epa_simplex2polytope.hpp:112-141
inline S2P simplex3(const MinkVertex& a, const MinkVertex& b, const MinkVertex& c, const MinkDiff& shape, Polytope& P,
                    V3& p0, V3& p1, double thr) {
  const V3 ab = b.vertex - a.vertex, ac = c.vertex - a.vertex;
  V3 n = cross(ab, ac);
  if (sqn(n) <= 0.0) return S2P::Failed;
  normalize(n);
  const V3 dir0 = n;
  const V3 d0 = shape.support(dir0);
  const double d0p = pointToPlane(d0, a.vertex, b.vertex, c.vertex);
  const V3 dir1 = -n;
  const V3 d1 = shape.support(dir1);
  const double d1p = pointToPlane(d1, a.vertex, b.vertex, c.vertex);
  if (d0p <= thr) { touchingPoint(shape, dir0, p0, p1); return S2P::Touching; }
  if (d1p <= thr) { touchingPoint(shape, dir1, p0, p1); return S2P::Touching; }
  MinkVertex dv;
  if (d0p > d1p) { dv.vertex = d0; dv.direction = dir0; }
  else { dv.vertex = d1; dv.direction = dir1; }
  return formTetra(a, b, c, dv, P);
}

// epa_simplex2polytope.hpp:176-376
inline S2P simplex2(const MinkVertex& a, const MinkVertex& b, const MinkDiff& shape, Polytope& P, V3& p0, V3& p1,
                    double thr) {
  const double thr2 = thr * thr;
  const V3 ab = b.vertex - a.vertex;
  if (sqn(ab) < thr2) return S2P::Failed;
  const V3 abu = normalized(ab);
  V3 dinit(abu[1], -abu[0], 0);
  bool ok = sqn(dinit) > thr2;
  if (!ok) { dinit = V3(abu[2], 0, -abu[0]); ok = sqn(dinit) > thr2; }
  if (!ok) { dinit = V3(0, abu[2], -abu[1]); ok = sqn(dinit) > thr2; }
  if (!ok) return S2P::Failed;
  normalize(dinit);
  const int kDiv = 72;
  V3 dcur = dinit, dfound, vfound;
  bool found = false;
  for (int i = 0; i < kDiv; ++i) {
    const V3 vcur = shape.support(dcur);
    const double dist = pointToLine(vcur, a.vertex, b.vertex);
    if (dist > thr) { vfound = vcur; dfound = dcur; found = true; break; }
    const double pi_value = 3.145926;  // the reference's constant, kept as is
    const double step = 2.0 * pi_value / kDiv;
    const V3 delta = cross(abu, vcur);
    dcur = dcur + step * delta;
    normalize(dcur);
  }
  if (!found) { touchingPoint(shape, dinit, p0, p1); return S2P::Touching; }
  MinkVertex v0{vfound, dfound};
  MinkVertex v1;
  v1.direction = -v0.direction;
  v1.vertex = shape.support(v1.direction);
  if (pointToLine(v1.vertex, a.vertex, b.vertex) < thr) { touchingPoint(shape, v1.direction, p0, p1); return S2P::Touching; }
  const V3 n = cross(v0.vertex - a.vertex, v1.vertex - a.vertex);
  if (sqn(n) < thr2) return S2P::Failed;
  MinkVertex v2;
  v2.direction = normalized(n);
  v2.vertex = shape.support(v2.direction);
  if (pointToLine(v2.vertex, a.vertex, b.vertex) < thr) { touchingPoint(shape, v2.direction, p0, p1); return S2P::Touching; }
  MinkVertex v3;
  v3.direction = -v2.direction;
  v3.vertex = shape.support(v3.direction);
  if (pointToLine(v3.vertex, a.vertex, b.vertex) < thr) { touchingPoint(shape, v3.direction, p0, p1); return S2P::Touching; }
  P.reset(P.face_capacity());
  int v[6] = {P.addVertex(a), P.addVertex(v0), P.addVertex(b), P.addVertex(v1), P.addVertex(v2), P.addVertex(v3)};
  int e[12] = {P.addEdge(v[0], v[1]), P.addEdge(v[1], v[2]), P.addEdge(v[2], v[3]), P.addEdge(v[3], v[0]),
               P.addEdge(v[4], v[0]), P.addEdge(v[4], v[1]), P.addEdge(v[4], v[2]), P.addEdge(v[4], v[3]),
               P.addEdge(v[5], v[0]), P.addEdge(v[5], v[1]), P.addEdge(v[5], v[2]), P.addEdge(v[5], v[3])};
  int f[8];
  f[0] = P.addFace(e[4], e[5], e[0]);
  f[1] = P.addFace(e[5], e[6], e[1]);
  f[2] = P.addFace(e[6], e[7], e[2]);
  f[3] = P.addFace(e[7], e[4], e[3]);
  f[4] = P.addFace(e[8], e[9], e[0]);
  f[5] = P.addFace(e[9], e[10], e[1]);
  f[6] = P.addFace(e[10], e[11], e[2]);
  f[7] = P.addFace(e[11], e[8], e[3]);
  for (int i = 0; i < 8; ++i) if (f[i] < 0) return S2P::Failed;
  return S2P::OK;
}

// epa_simplex2polytope.hpp:41-110
inline S2P simplexToPolytope(const Simplex& s, const MinkDiff& shape, Polytope& P, V3& p0, V3& p1, double thr) {
  const double thr2 = thr * thr;
  for (int i = 0; i < s.rank; ++i) {
    if (sqn(s.v[i].vertex) <= thr2) { touchingPoint(shape, s.v[i].direction, p0, p1); return S2P::Touching; }
  }
  if (s.rank == 4) {
    const MinkVertex &a = s.v[0], &b = s.v[1], &c = s.v[2], &d = s.v[3];
    const V3 o;
    if (pointToPlane(o, a.vertex, b.vertex, c.vertex) < thr) return simplex3(a, b, c, shape, P, p0, p1, thr);
    if (pointToPlane(o, a.vertex, c.vertex, d.vertex) < thr) return simplex3(a, c, d, shape, P, p0, p1, thr);
    if (pointToPlane(o, a.vertex, b.vertex, d.vertex) < thr) return simplex3(a, b, d, shape, P, p0, p1, thr);
    if (pointToPlane(o, b.vertex, c.vertex, d.vertex) < thr) return simplex3(b, c, d, shape, P, p0, p1, thr);
    return formTetra(a, b, c, d, P);
  }
  if (s.rank == 3) return simplex3(s.v[0], s.v[1], s.v[2], shape, P, p0, p1, thr);
  if (s.rank == 2) return simplex2(s.v[0], s.v[1], shape, P, p0, p1, thr);
  const V3& d = s.v[0].direction;
  p0 = shape.support0(d);
  p1 = shape.support1(-d);
  return S2P::Touching;
}

class EPA {
 public:
  EPA(size_t max_faces, int max_iter, double tol) : max_faces_(max_faces), max_iter_(max_iter), tol_(tol) {}
  int iterations = 0;

  // epa.hpp:239-257 (Evaluate) + :115-131 (from uninitialised polytope)
  EPAStatus Evaluate(const Simplex& s, const MinkDiff& shape, double& depth, V3& p0, V3& p1) {
    iterations = 0;
    Polytope P(max_faces_);
    const S2P st = simplexToPolytope(s, shape, P, p0, p1, tol_);
    if (st == S2P::Failed) return EPAStatus::Failed;
    if (st == S2P::Touching) { depth = 0.0; return EPAStatus::Touching; }
    return fromPolytope(P, shape, depth, p0, p1);
  }

 private:
  size_t max_faces_;
  int max_iter_;
  double tol_;
  struct Raw {
    FeatType type = FeatType::None;
    MinDist md;
    MinkVertex a, b, c;
  };
  enum class Dir { OK, Failed, Converge };

  // epa.hpp:10-113
  Dir nextDirection(const Polytope& P, const MinkDiff& shape, FeatType ft, int fi, V3& nd, V3& nv, int& start) const {
    const double thr = 1e-3 * 1e-3;
    auto face_cand = [&](int f, bool try_witness) -> Dir {
      V3 fn;
      if (!P.faceNormalOut(f, fn, nullptr)) return Dir::Failed;
      const V3& onf = P.V[P.E[P.F[f].e[0]].v[0]].loc;
      const MinDist& md = P.F[f].md;
      if (try_witness && md.sq > thr) {
        nd = normalized(md.w);
        nv = shape.support(nd);
        if (dot(fn, nv - onf) >= 0.0) { start = f; return Dir::OK; }
      }
      nd = fn;
      nv = shape.support(nd);
      if (dot(fn, nv - onf) > tol_) { start = f; return Dir::OK; }
      return Dir::Converge;
    };
    if (ft == FeatType::Face) return face_cand(fi, true);
    if (ft == FeatType::Edge) {
      const Polytope::PE& e = P.E[fi];
      const int f0 = e.f[0], f1 = e.f[1];
      if (f0 < 0 || f1 < 0) return Dir::Failed;  // an open edge would be a null face in the reference
      if (e.md.sq > thr) {
        nd = normalized(e.md.w);
        nv = shape.support(nd);
        if (P.pointOutside(f0, nv)) { start = f0; return Dir::OK; }
        if (P.pointOutside(f1, nv)) { start = f1; return Dir::OK; }
      }
      const Dir s0 = face_cand(f0, false);
      if (s0 == Dir::OK) return s0;
      return face_cand(f1, false);
    }
    return Dir::Failed;
  }

  // epa.hpp:300-338
  static void toRaw(const Polytope& P, FeatType ft, int i, Raw& r) {
    r.type = ft;
    if (ft == FeatType::Edge) {
      const Polytope::PE& e = P.E[i];
      r.md = e.md;
      r.a = {P.V[e.v[0]].loc, P.V[e.v[0]].dir};
      r.b = {P.V[e.v[1]].loc, P.V[e.v[1]].dir};
    } else {
      r.md = P.F[i].md;
      int a, b, c;
      P.faceVerts(i, a, b, c);
      r.a = {P.V[a].loc, P.V[a].dir};
      r.b = {P.V[b].loc, P.V[b].dir};
      r.c = {P.V[c].loc, P.V[c].dir};
    }
  }

  // epa.hpp:268-299
  bool terminate(const Raw& r, const V3& nv) const {
    double dsq = 0.0;
    if (r.type == FeatType::Edge) {
      bool in = false;
      pointToSegment(nv, r.a.vertex, r.b.vertex, in, dsq, nullptr);
    } else {
      const double pp = pointToPlane(nv, r.a.vertex, r.b.vertex, r.c.vertex);
      dsq = pp * pp;
    }
    return dsq < tol_ * tol_;
  }

  // epa.hpp:425-498
  static bool pairFromFace(const MinkDiff& shape, const Raw& r, double& depth, V3& p0, V3& p1) {
    depth = std::sqrt(r.md.sq);
    const V3 &a = r.a.vertex, &b = r.b.vertex, &c = r.c.vertex;
    const V3& p = r.md.w;
    const V3 dl0 = a - b, dl1 = b - c, dl2 = c - a;
    const V3 n = cross(dl0, dl1);
    const double area = std::sqrt(sqn(n));
    double w[3];
    w[0] = norm(cross(dl1, b - p)) / area;
    w[1] = norm(cross(dl2, c - p)) / area;
    const double chk = norm(cross(dl0, a - p)) / area;
    w[2] = 1.0 - w[0] - w[1];
    if (std::abs(chk - w[2]) > 0.01) return false;
    p0 = (w[0] * shape.support0(r.a.direction) + w[1] * shape.support0(r.b.direction)) + w[2] * shape.support0(r.c.direction);
    p1 = (w[0] * shape.support1(-r.a.direction) + w[1] * shape.support1(-r.b.direction)) + w[2] * shape.support1(-r.c.direction);
    return true;
  }
  // epa.hpp:367-423
  static bool pairFromSegment(const MinkDiff& shape, const Raw& r, double& depth, V3& p0, V3& p1) {
    depth = std::sqrt(r.md.sq);
    const V3& p = r.md.w;
    const V3 &a = r.a.vertex, &b = r.b.vertex;
    const V3 ab = b - a;
    int k = 0;
    double m = std::abs(ab[0]);
    if (std::abs(ab[1]) > m) { k = 1; m = std::abs(ab[1]); }
    if (std::abs(ab[2]) > m) { k = 2; m = std::abs(ab[2]); }
    if (m <= 1e-10) {
      p0 = shape.support0(r.a.direction);
      p1 = shape.support1(-r.a.direction);
      return true;
    }
    const double s = (p[k] - a[k]) / (b[k] - a[k]);
    if (s < 0 || s > 1.0) return false;
    const double wa = 1.0 - s, wb = s;
    p0 = wa * shape.support0(r.a.direction) + wb * shape.support0(r.b.direction);
    p1 = wa * shape.support1(-r.a.direction) + wb * shape.support1(-r.b.direction);
    return true;
  }
  // epa.hpp:340-365
  static void assignPair(const MinkDiff& shape, const MinkVertex& cand, const Raw& r, double& depth, V3& p0, V3& p1) {
    if (r.type == FeatType::Edge) {
      if (pairFromSegment(shape, r, depth, p0, p1)) return;
    } else if (r.type == FeatType::Face) {
      if (pairFromFace(shape, r, depth, p0, p1)) return;
    }
    p0 = shape.support0(cand.direction);
    p1 = shape.support1(-cand.direction);
    depth = norm(p0 - p1);
  }

  // epa.hpp:133-237
  EPAStatus fromPolytope(Polytope& P, const MinkDiff& shape, double& depth, V3& p0, V3& p1) {
    int iteration = 0;
    Raw raw;
    while (true) {
      int idx;
      FeatType ft = P.nearest(false, idx);
      if (ft == FeatType::None) return EPAStatus::Failed;
      if (ft == FeatType::Vertex) {
        const double vsq = P.V[idx].md.sq;
        const double ratio = 1.0 - 1e-3;
        int oidx;
        const FeatType ot = P.nearest(true, oidx);
        if (ot == FeatType::None) return EPAStatus::Failed;
        if (ot == FeatType::Edge) {
          if (ratio * P.E[oidx].md.sq < vsq) { ft = ot; idx = oidx; }
        } else if (ot == FeatType::Face) {
          if (ratio * P.F[oidx].md.sq < vsq) { ft = ot; idx = oidx; }
        }
      }
      if (ft != FeatType::Edge && ft != FeatType::Face) return EPAStatus::Failed;
      toRaw(P, ft, idx, raw);
      V3 nd, nv;
      int start = -1;
      const Dir ds = nextDirection(P, shape, ft, idx, nd, nv, start);
      if (ds == Dir::Failed) return EPAStatus::Failed;
      if (ds == Dir::Converge) {
        assignPair(shape, {nv, nd}, raw, depth, p0, p1);
        return EPAStatus::OK;
      }
      if (start < 0) return EPAStatus::Failed;
      const MinkVertex nxt{nv, nd};
      if (terminate(raw, nv)) {
        assignPair(shape, nxt, raw, depth, p0, p1);
        return EPAStatus::OK;
      }
      const Polytope::Expand es = P.expand(nxt, start);
      if (es == Polytope::Expand::Failed) return EPAStatus::Failed;
      if (es == Polytope::Expand::MallocFailed) {
        assignPair(shape, nxt, raw, depth, p0, p1);
        return EPAStatus::MallocFailed;
      }
      iteration += 1;
      iterations = iteration;
      if (iteration >= max_iter_) {
        assignPair(shape, nxt, raw, depth, p0, p1);
        return EPAStatus::IterationLimit;
      }
    }
  }
};

// -------------------------------------------------------------------- MPR --
enum class MPRStatus : int { Intersect = 0, Separated = 1, Failed = 2 };

// MPR::IntersectData (mpr.h:23-31) as the run leaves it: the interior point,
// the portal and the directions that found its vertices; `count` = how many
// of v1..v3 were set (the reference leaves the others NaN).
struct MPRPortal {
  V3 v0, v[3], d[3];
  int count = 0;
};

class MPR {
 public:
  MPR(int max_iter, double tol) : max_iter_(max_iter), tol_(tol) {}

  // mpr.hpp:33-185
  MPRStatus Intersect(const MinkDiff& shape, MPRPortal* keep = nullptr) const {
    V3 v0 = shape.interior();
    V3 d1, d2, d3, v1, v2, v3;
    int count = 0;
    const MPRStatus st = run(shape, v0, v1, v2, v3, d1, d2, d3, count);
    if (keep) {
      keep->v0 = v0;
      keep->v[0] = v1; keep->v[1] = v2; keep->v[2] = v3;
      keep->d[0] = d1; keep->d[1] = d2; keep->d[2] = d3;
      keep->count = count;
    }
    return st;
  }

 private:
  MPRStatus run(const MinkDiff& shape, const V3& v0, V3& v1, V3& v2, V3& v3, V3& d1, V3& d2, V3& d3,
                int& count) const {
    if (sqn(v0) <= tol_ * tol_) return MPRStatus::Intersect;
    d1 = -v0;
    v1 = sup(shape, d1);
    count = 1;
    if (dot(d1, v1) < 0) return MPRStatus::Separated;
    d2 = cross(v0, v1);
    if (absnorm(d2) <= absnorm(v0) * absnorm(v1) * tol_) return MPRStatus::Intersect;
    v2 = sup(shape, d2);
    count = 2;
    if (dot(d2, v2) < 0) return MPRStatus::Separated;
    d3 = cross(v1 - v0, v2 - v0);
    if (dot(d3, v0) > 0) {
      std::swap(v1, v2);
      std::swap(d1, d2);
      d3 = -d3;
    }
    v3 = sup(shape, d3);
    count = 3;
    if (dot(d3, v3) < 0) return MPRStatus::Separated;
    const int fp = findPortal(shape, v0, v1, v2, v3, d1, d2, d3);
    if (fp == 0) return MPRStatus::Failed;
    if (fp == 1) return MPRStatus::Separated;
    int it = 0;
    while (it < max_iter_) {
      it += 1;
      V3 n = cross(v2 - v1, v3 - v1);
      if (dot(n, v0) > 0) {
        std::swap(v2, v3);
        std::swap(d2, d3);
        n = -n;
      }
      if (!(dot(v1, n) < 0)) return MPRStatus::Intersect;
      const V3 v4 = sup(shape, n);
      if (dot(v4, n) < 0) return MPRStatus::Separated;
      if (std::abs(dot(v4 - v1, n)) < tol_ * absnorm(n)) return MPRStatus::Separated;
      updatePortal(v0, v4, n, v1, v2, v3, d1, d2, d3);
    }
    return MPRStatus::Failed;
  }

 private:
  int max_iter_;
  double tol_;
  static constexpr double kEps = std::numeric_limits<double>::epsilon();

  // mpr.hpp:10-15: normalises the direction in place, then supports.
  static V3 sup(const MinkDiff& shape, V3& d) {
    normalize(d);
    return shape.support(d);
  }
  // mpr.hpp:187-328; returns 0 iteration limit, 1 separated, 2 portal found
  int findPortal(const MinkDiff& shape, const V3& v0, V3& v1, V3& v2, V3& v3, V3& d1, V3& d2, V3& d3) const {
    const double v0n = absnorm(v0);
    int it = 0;
    while (true) {
      if (it >= max_iter_) return 0;
      it += 1;
      V3 a1 = v1 - v0, a2 = v2 - v0, a3 = v3 - v0;
      V3 n031 = cross(a3, a1);
      V3 n012 = cross(a1, a2);
      const double vol = dot(a2, n031);
      if (vol < 0) {
        std::swap(v2, v3);
        std::swap(d2, d3);
        std::swap(a2, a3);
        std::swap(n012, n031);
        n031 = -n031;
        n012 = -n012;
      }
      if (dot(v0, n031) > kEps * v0n * absnorm(n031)) {
        V3 sd = -n031;
        v2 = sup(shape, sd);
        d2 = sd;
        if (dot(v2, sd) < 0) return 1;
        continue;
      }
      if (dot(v0, n012) > kEps * v0n * absnorm(n012)) {
        V3 sd = -n012;
        v3 = sup(shape, sd);
        d3 = sd;
        if (dot(v3, sd) < 0) return 1;
        continue;
      }
      V3 n023 = cross(a2, a3);
      if (dot(v0, n023) > kEps * v0n * absnorm(n023)) {
        V3 sd = -n023;
        v1 = sup(shape, sd);
        d1 = sd;
        if (dot(v1, sd) < 0) return 1;
        continue;
      }
      return 2;
    }
  }
 public:
  // ------------------------------------------------------------------
  // Directed penetration, mpr.hpp:495-595 (RunDirectedPenetration) and
  // :606-701 (finalizeDirectedPenetrationResult): the depth of the Minkowski
  // difference along the unit direction d (shape 1's escape direction in
  // shape 0's frame), with witness points p0 / p1 in shape 0's frame.
  // Status: 0 OK, 1 Failed, 2 FailedNoIntersect, 3 FailedRefinementIterationLimit.
  struct Directed {
    V3 v1, v2, v3, d1, d2, d3, portal_normal, p0, p1;
    double distance = 0;
  };
  int DirectedPenetration(const MinkDiff& shape, const V3& d, Directed& pd) const {
    const V3 v0 = -d;
    V3 &v1 = pd.v1, &v2 = pd.v2, &v3 = pd.v3, &d1 = pd.d1, &d2 = pd.d2, &d3 = pd.d3;
    d1 = d;
    v1 = sup(shape, d1);
    if (dot(d1, v1) < 0) return 2;
    d2 = cross(v0, v1);
    if (absnorm(d2) <= absnorm(v1) * tol_) {
      pd.distance = dot(v1, d);
      pd.portal_normal = d1;
      pd.p0 = shape.support0(d1);
      pd.p1 = shape.support1(-d1);
      return 0;
    }
    v2 = sup(shape, d2);
    if (dot(d2, v2) < 0) return 2;
    d3 = cross(v1, v2);
    if (dot(d3, v0) > 0) {
      std::swap(v1, v2);
      std::swap(d1, d2);
      d3 = -d3;
    }
    v3 = sup(shape, d3);
    if (dot(d3, v3) < 0) return 2;
    const double m2 = std::max(sqn(v1), std::max(sqn(v2), sqn(v3)));
    const V3 v0s = v0 * std::sqrt(m2);
    const int fp = findPortal(shape, v0s, v1, v2, v3, d1, d2, d3);
    if (fp == 0) return 1;
    if (fp == 1) return 2;
    for (int it = 0; it < max_iter_; ++it) {
      V3 n = cross(v2 - v1, v3 - v1);
      if (dot(n, d) < 0) {
        std::swap(v2, v3);
        std::swap(d2, d3);
        n = -n;
      }
      const V3 v4 = sup(shape, n);
      if (dot(v4, n) < 0) return 2;
      if (std::abs(dot(v4 - v1, n)) < tol_ * absnorm(n)) {
        finalizeDirected(shape, d, n, pd, &v4);
        return 0;
      }
      updatePortal(v0s, v4, n, v1, v2, v3, d1, d2, d3);
    }
    return 3;
  }

 public:
  // ------------------------------------------------------------------
  // Incremental minimum-distance penetration (fcl::collide with
  // useIncrementalMinimumDistancePenetration, collision_penetration-inl.h:133-155):
  // mpr_incremental_penetration.hpp:176-288 (RunIncrementalMinimumPenetrationDistance,
  // return_on_subroutine_converge = true), :49-174 (the explore subroutine),
  // :10-47 (the distance bounds along the ray) and :300-333 (the witness
  // points).  Status: 0 OK, 1 Failed, 2 FailedNoIntersect, 4 IterationLimit.
  struct Incremental {
    double depth = 0;
    V3 dir, p0, p1;
  };
  int IncrementalPenetration(const MinkDiff& shape, const V3& init_direction, Incremental& out) const {
    V3 d = init_direction;
    V3 v1, v2, v3, d1, d2, d3;
    V3 prev_dir = init_direction;
    double prev_lb = -1, prev_ub = -1;
    for (int outer = 0; outer < max_iter_; ++outer) {
      V3 nd;
      double lb = 0, ub = 0;
      const int st = explore(shape, d, v1, v2, v3, d1, d2, d3, lb, ub, nd, outer >= 1);
      if (st == 0) {
        d = nd;
      } else if (st == 1) {
        finalizeIncremental(shape, d, v1, v2, v3, d1, d2, d3, lb, ub, out);
        return 0;
      } else if (st == 2) {
        out.depth = ub;
        out.dir = nd;
        out.p0 = shape.support0(nd);
        out.p1 = shape.support1(-nd);
        return 0;
      } else if (st == 4) {
        return 2;
      } else {
        return 1;
      }
      prev_dir = nd;
      prev_lb = lb;
      prev_ub = ub;
    }
    (void)prev_dir;
    finalizeIncremental(shape, d, v1, v2, v3, d1, d2, d3, prev_lb, prev_ub, out);
    return 4;
  }

 private:
  // explore subroutine status: 0 NewDirection, 1 SubroutineConverge,
  // 2 Degenerated, 3 Failed, 4 FailedNoIntersect
  int explore(const MinkDiff& shape, const V3& d, V3& v1, V3& v2, V3& v3, V3& d1, V3& d2, V3& d3, double& lb,
              double& ub, V3& nd, bool v123_valid) const {
    const V3 v0 = -d;
    V3 init_dir = d;
    const V3 init = sup(shape, init_dir);
    if (dot(d, init) < 0) return 4;
    if (!v123_valid) {
      d1 = d;
      v1 = init;
      d2 = cross(v0, v1);
      if (absnorm(d2) <= absnorm(v1) * tol_) {
        lb = dot(v1, d);
        ub = lb;
        nd = d;
        return 2;
      }
      v2 = sup(shape, d2);
      if (dot(d2, v2) < 0) return 4;
      d3 = cross(v1, v2);
      if (dot(d3, v0) > 0) {
        std::swap(v1, v2);
        std::swap(d1, d2);
        d3 = d3 * -1.0;
      }
      v3 = sup(shape, d3);
      if (dot(d3, v3) < 0) return 4;
    }
    V3 v0s = v0;
    {
      const double m2 = std::max(sqn(v1), std::max(sqn(v2), sqn(v3)));
      v0s = v0s * std::sqrt(m2);
    }
    const int fp = findPortal(shape, v0s, v1, v2, v3, d1, d2, d3);
    if (fp == 0) return 3;
    if (fp == 1) return 4;
    int it = 0;
    while (it < max_iter_) {
      it += 1;
      V3 n = cross(v2 - v1, v3 - v1);
      if (dot(n, d) < 0) {
        std::swap(v2, v3);
        std::swap(d2, d3);
        n = n * -1.0;
      }
      const V3 v4 = sup(shape, n);
      const double ub_plane = dot(v4, n);
      if (ub_plane < 0) return 4;
      const double v1n = dot(v1, n), v4n = dot(v4, n);
      const double v14 = v4n - v1n;
      const double ndd = dot(d, n);
      if (std::abs(ndd) <= 0) {
        lb = std::max(dot(v1, d), std::max(dot(v2, d), dot(v3, d)));
        ub = lb;
      } else {
        lb = v1n / ndd;
        ub = v4n / ndd;
      }
      if (lb > ub_plane + tol_) {
        nd = n;
        return 0;
      }
      if (std::abs(v14) <= tol_) {
        nd = n;
        return 1;
      }
      updatePortal(v0s, v4, n, v1, v2, v3, d1, d2, d3);
    }
    return 3;
  }

  static void finalizeIncremental(const MinkDiff& shape, const V3& d, const V3& v1, const V3& v2, const V3& v3,
                                  const V3& d1, const V3& d2, const V3& d3, double lb, double ub, Incremental& out) {
    out.depth = ub;
    out.dir = d;
    const V3 o_projected = d * lb;
    const V3 a12 = v2 - v1, a13 = v3 - v1;
    const double area = norm(cross(a12, a13));
    const double w2 = norm(cross(a13, v1 - o_projected)) / area;
    const double w3 = norm(cross(a12, v1 - o_projected)) / area;
    const double w1 = 1.0 - w2 - w3;
    out.p0 = (shape.support0(d1) * w1 + shape.support0(d2) * w2) + shape.support0(d3) * w3;
    out.p1 = (shape.support1(-d1) * w1 + shape.support1(-d2) * w2) + shape.support1(-d3) * w3;
  }

  static void finalizeDirected(const MinkDiff& shape, const V3& d, const V3& n, Directed& pd, const V3* v4) {
    pd.portal_normal = n;
    const double ndd = dot(d, n);
    if (std::abs(ndd) <= 0) {
      const double dv[3] = {dot(pd.v1, d), dot(pd.v2, d), dot(pd.v3, d)};
      const V3* dirs[3] = {&pd.d1, &pd.d2, &pd.d3};
      double best = -std::numeric_limits<double>::infinity();
      int bi = 0;
      for (int i = 0; i < 3; ++i)
        if (dv[i] > best) { best = dv[i]; bi = i; }
      pd.distance = best;
      pd.p0 = shape.support0(*dirs[bi]);
      pd.p1 = shape.support1(-*dirs[bi]);
      return;
    }
    const double dist_to_v123 = dot(pd.v1, n) / ndd;
    pd.distance = v4 ? dot(*v4, n) / ndd : dist_to_v123;
    const V3 o_projected = d * dist_to_v123;
    const V3 a12 = pd.v2 - pd.v1, a13 = pd.v3 - pd.v1;
    const double area = norm(cross(a12, a13));
    const double w2 = norm(cross(a13, pd.v1 - o_projected)) / area;
    const double w3 = norm(cross(a12, pd.v1 - o_projected)) / area;
    const double w1 = 1.0 - w2 - w3;
    pd.p0 = (shape.support0(pd.d1) * w1 + shape.support0(pd.d2) * w2) + shape.support0(pd.d3) * w3;
    pd.p1 = (shape.support1(-pd.d1) * w1 + shape.support1(-pd.d2) * w2) + shape.support1(-pd.d3) * w3;
  }

 public:
  // mpr.hpp:434-493
  static void updatePortal(const V3& v0, const V3& v4, const V3& n, V3& v1, V3& v2, V3& v3, V3& d1, V3& d2, V3& d3) {
    const V3 pn = cross(v4, v0);
    if (dot(v1, pn) > 0) {
      if (dot(v2, pn) > 0) { v1 = v4; d1 = n; }
      else { v3 = v4; d3 = n; }
    } else {
      if (dot(v3, pn) > 0) { v2 = v4; d2 = n; }
      else { v1 = v4; d1 = n; }
    }
  }
};

// ------------------------------------------------------------ the bridge --
// GJKSolver defaults (gjk_solver-inl.h:1120-1130) as fcl::collide sets them
// from CollisionRequest (collision_interface-inl.h:18-20,
// collision_request-inl.h:54-60): GJK 128 iterations / 1e-6, EPA 256 faces,
// 255 iterations, 1e-6.
struct SolverParams {
  int gjk_max_iter = 128;
  double gjk_tol = 1e-6;
  size_t epa_max_faces = 256;
  int epa_max_iter = 255;
  double epa_tol = 1e-6;
};

struct QueryOut {
  bool ok = false;       // shapeSignedDistance's return value / collide flag
  double distance = -1;  // signed distance (>0 separation, <0 -depth)
  V3 p0, p1;             // witness points in shape 0's frame
  int gjk_status = -1;
  int epa_status = -1;
  int gjk_iters = 0;
  int epa_iters = 0;
};

// ShapeSignedDistanceIndepImpl::run, gjk_solver-inl.h:810-863.
inline QueryOut signedDistance(const MinkDiff& md, const SolverParams& sp, const V3* guess) {
  QueryOut o;
  V3 g(1, 0, 0);
  if (guess) g = *guess;
  GJK gjk(sp.gjk_max_iter, sp.gjk_tol);
  Simplex s;
  MinDistOut mdo;
  const GJKStatus gs = gjk.Evaluate(md, s, -g, &mdo);
  o.gjk_status = (int)gs;
  o.gjk_iters = gjk.iterations;
  if (gs == GJKStatus::Separated && mdo.point_valid) {
    o.ok = true;
    o.p0 = mdo.p0;
    o.p1 = mdo.p1;
    o.distance = norm(mdo.p0 - mdo.p1);
    return o;
  }
  if (gs == GJKStatus::Intersect) {
    EPA epa(sp.epa_max_faces, sp.epa_max_iter, sp.epa_tol);
    double depth = 0;
    V3 p0, p1;
    const EPAStatus es = epa.Evaluate(s, md, depth, p0, p1);
    o.epa_status = (int)es;
    o.epa_iters = epa.iterations;
    if (es != EPAStatus::Failed) {
      o.ok = true;
      o.p0 = p0;
      o.p1 = p1;
      o.distance = -depth;
    }
    return o;
  }
  o.distance = -1;
  return o;
}

// ShapeIntersectIndepImpl::run, gjk_solver-inl.h:70-137: boolean collide
// (MPR first, GJK when MPR fails) or, when contacts are requested, GJK then
// EPA, reporting EPA failure as "no collision".
inline QueryOut intersect(const MinkDiff& md, const SolverParams& sp, bool want_contact, const V3* guess) {
  QueryOut o;
  V3 g(1, 0, 0);
  if (guess) g = *guess;
  if (!want_contact) {
    MPR mpr(sp.gjk_max_iter, sp.gjk_tol);
    const MPRStatus ms = mpr.Intersect(md);
    if (ms == MPRStatus::Intersect) { o.ok = true; o.gjk_status = 10; return o; }
    if (ms == MPRStatus::Separated) { o.ok = false; o.gjk_status = 11; return o; }
  }
  GJK gjk(sp.gjk_max_iter, sp.gjk_tol);
  Simplex s;
  const GJKStatus gs = gjk.Evaluate(md, s, -g, nullptr);
  o.gjk_status = (int)gs;
  o.gjk_iters = gjk.iterations;
  if (!want_contact) { o.ok = (gs == GJKStatus::Intersect); return o; }
  if (gs != GJKStatus::Intersect) { o.ok = false; return o; }
  EPA epa(sp.epa_max_faces, sp.epa_max_iter, sp.epa_tol);
  double depth = 0;
  V3 p0, p1;
  const EPAStatus es = epa.Evaluate(s, md, depth, p0, p1);
  o.epa_status = (int)es;
  o.epa_iters = epa.iterations;
  if (es == EPAStatus::Failed) { o.ok = false; return o; }
  o.ok = true;
  o.p0 = p0;
  o.p1 = p1;
  o.distance = -depth;
  return o;
}

}  // namespace orc
