// ORACLE — test infrastructure only.
//
// Driver that runs the reference's own GJK / EPA / MPR (include/fcl/cvx_collide/,
// compiled unmodified through oracle/eigen_shim) on the packed shape / pair
// buffers the GPU library and the FP64 restatement take.  oracle/build_ref.sh
// builds it into oracle/_ref/libfcl_ref.so; it needs the reference sources and
// is therefore only built where they exist.  Tests use it to pin the
// restatement bit for bit.
//
// The few pieces restated here because they live in headers that need the
// whole fcl geometry stack: the Convex naive support scan
// (include/fcl/geometry/shape/convex-inl.h:133-149) and interior point
// (convex-inl.h:58-63), and the GJKSolver bridge policies
// ShapeSignedDistanceIndepImpl (gjk_solver-inl.h:810-863) and
// ShapeIntersectIndepImpl (gjk_solver-inl.h:70-137).
#include <cmath>
#include <cstdint>
#include <limits>
#include <thread>
#include <vector>

#include "fcl/cvx_collide/epa.h"
#include "fcl/cvx_collide/gjk.h"
#include "fcl/cvx_collide/mpr.h"

using namespace fcl::cvx_collide;
using Vec = Vector3<double>;

namespace {

struct ShapeRec {
  int32_t type;
  uint32_t vert_offset, vert_count, reserved;
  float param[4];
};
struct PairRec {
  uint32_t shape_a, shape_b;
  float rot[9];
  float trans[3];
  uint32_t flags, reserved;
};
struct ConvexData {
  const float* v;
  int n;
  Vec mean;
};

Vec supportFn(const GJKGeometryData<double>& g, const Vec& d) {
  if (g.shape_type == GJKShapeType::ShapeSweptVolume) {
    // computeSupport's swept-volume case (narrowphase/detail/gjk_solver_cvx-inl.h:93-101)
    const Vec p = supportFn(*static_cast<const GJKGeometryData<double>*>(g.user_ptr), d);
    return (d.dot(g.vec3_data) > 0) ? Vec(p + g.vec3_data) : p;
  }
  if (g.shape_type == GJKShapeType::Convex) {
    const ConvexData* c = static_cast<const ConvexData*>(g.user_ptr);
    int best = 0;
    double best_val = d.dot(Vec(c->v[0], c->v[1], c->v[2]));
    for (int i = 1; i < c->n; ++i) {
      const double val = d.dot(Vec(c->v[4 * i], c->v[4 * i + 1], c->v[4 * i + 2]));
      if (val > best_val) { best = i; best_val = val; }
    }
    return Vec(c->v[4 * best], c->v[4 * best + 1], c->v[4 * best + 2]);
  }
  return basicGeometrySupport<double>(g, d);
}

Vec interiorFn(const GJKGeometryData<double>& g) {
  if (g.shape_type == GJKShapeType::ShapeSweptVolume)  // gjk_solver_cvx-inl.h:131-138
    return Vec(interiorFn(*static_cast<const GJKGeometryData<double>*>(g.user_ptr)) + 0.5 * g.vec3_data);
  if (g.shape_type == GJKShapeType::Convex) return static_cast<const ConvexData*>(g.user_ptr)->mean;
  return basicGeometryInterior<double>(g);
}

struct Prepared {
  std::vector<GJKGeometryData<double>> geo;
  std::vector<ConvexData> cvx;
};

Prepared prepare(const ShapeRec* s, int n, const float* verts) {
  Prepared p;
  p.geo.resize((size_t)n);
  p.cvx.resize((size_t)n);
  for (int i = 0; i < n; ++i) {
    GJKGeometryData<double>& g = p.geo[(size_t)i];
    switch (s[i].type) {
      case 0: g = constructGJKBox<double>(Vec(s[i].param[0], s[i].param[1], s[i].param[2])); break;
      case 1: g = constructGJKSphere<double>(s[i].param[0]); break;
      case 3: g = constructGJKCapsule<double>(s[i].param[0], s[i].param[1]); break;
      case 5: g = constructGJKCylinder<double>(s[i].param[0], s[i].param[1]); break;
      default: {
        ConvexData& c = p.cvx[(size_t)i];
        c.v = verts + 4 * (size_t)s[i].vert_offset;
        c.n = (int)s[i].vert_count;
        Vec sum = Vec::Zero();
        for (int k = 0; k < c.n; ++k) sum += Vec(c.v[4 * k], c.v[4 * k + 1], c.v[4 * k + 2]);
        c.mean = sum * (double)(1.0 / (double)c.n);
        g.shape_type = GJKShapeType::Convex;
        g.user_ptr = &c;
      }
    }
  }
  return p;
}

MinkowskiDiff<double> makeDiff(const Prepared& p, const PairRec& pr) {
  MinkowskiDiff<double> md;
  md.shapes[0] = p.geo[pr.shape_a];
  md.shapes[1] = p.geo[pr.shape_b];
  md.support_function = supportFn;
  md.interior_function = interiorFn;
  Transform3<double> to0;
  to0.setIdentity();
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) to0.linear()(r, c) = pr.rot[3 * r + c];
  to0.translation() = Vec(pr.trans[0], pr.trans[1], pr.trans[2]);
  md.toshape0 = to0;
  md.toshape1 = to0.linear().transpose();
  return md;
}

template <typename F>
void parallelFor(int n, int nt, F&& f) {
  if (nt <= 1 || n < 2 * nt) { f(0, n); return; }
  std::vector<std::thread> th;
  const int chunk = (n + nt - 1) / nt;
  for (int t = 0; t < nt; ++t) {
    const int b = t * chunk, e = std::min(n, b + chunk);
    if (b >= e) break;
    th.emplace_back([&f, b, e] { f(b, e); });
  }
  for (auto& x : th) x.join();
}

}  // namespace

extern "C" {

struct RefResult {  // same layout as the restatement's OrcResult
  double distance, p0[3], p1[3], normal[3];
  int32_t ok, gjk_status, epa_status, gjk_iters, epa_iters, reserved;
};

static void finish(RefResult& r, bool contact) {
  Vec p0(r.p0[0], r.p0[1], r.p0[2]), p1(r.p1[0], r.p1[1], r.p1[2]);
  Vec n = (r.ok && r.distance > 0 && !contact) ? Vec(p1 - p0) : Vec(p0 - p1);
  if (n.squaredNorm() <= 0) n = Vec(0, 0, 1);
  else n.normalize();
  for (int k = 0; k < 3; ++k) r.normal[k] = n[k];
}

int ref_signed_distance(const void* shapes, int n_shapes, const float* verts, const void* pairs, int n_pairs,
                        const float* guess, RefResult* out, int n_threads, int gjk_max_iter, double gjk_tol) {
  if (gjk_max_iter <= 0) gjk_max_iter = 128;
  if (gjk_tol <= 0) gjk_tol = 1e-6;
  const Prepared p = prepare((const ShapeRec*)shapes, n_shapes, verts);
  const PairRec* pr = (const PairRec*)pairs;
  parallelFor(n_pairs, n_threads, [&](int b, int e) {
    for (int i = b; i < e; ++i) {
      RefResult& r = out[i];
      r = RefResult{};
      r.distance = -1;
      r.epa_status = -1;
      const MinkowskiDiff<double> md = makeDiff(p, pr[i]);
      Vec g(1, 0, 0);
      if (guess) g = Vec(guess[3 * i], guess[3 * i + 1], guess[3 * i + 2]);
      GJK<double> gjk(gjk_max_iter, gjk_tol);
      GJKSimplex<double> s;
      GJK<double>::MinSeparationDistanceOutput mdo;
      const GJK_Status gs = gjk.Evaluate(md, s, -g, &mdo);
      r.gjk_status = (int)gs;
      if (gs == GJK_Status::Separated && mdo.is_separation_point_valid) {
        r.ok = 1;
        for (int k = 0; k < 3; ++k) { r.p0[k] = mdo.p0_if_separated[k]; r.p1[k] = mdo.p1_if_separated[k]; }
        r.distance = mdo.separation_distance();
      } else if (gs == GJK_Status::Intersect) {
        EPA<double> epa(256, 255, 1e-6);
        double depth = 0;
        Vec a, bb;
        const EPA_Status es = epa.Evaluate(s, md, &depth, &a, &bb);
        r.epa_status = (int)es;
        if (es != EPA_Status::Failed) {
          r.ok = 1;
          for (int k = 0; k < 3; ++k) { r.p0[k] = a[k]; r.p1[k] = bb[k]; }
          r.distance = -depth;
        }
      }
      finish(r, false);
    }
  });
  return 0;
}

int ref_collide(const void* shapes, int n_shapes, const float* verts, const void* pairs, int n_pairs,
                int want_contact, RefResult* out, int n_threads) {
  const Prepared p = prepare((const ShapeRec*)shapes, n_shapes, verts);
  const PairRec* pr = (const PairRec*)pairs;
  parallelFor(n_pairs, n_threads, [&](int b, int e) {
    for (int i = b; i < e; ++i) {
      RefResult& r = out[i];
      r = RefResult{};
      r.distance = -1;
      r.epa_status = -1;
      const MinkowskiDiff<double> md = makeDiff(p, pr[i]);
      if (!want_contact) {
        MPR<double> mpr(128, 1e-6);
        const auto ms = mpr.Intersect(md);
        if (ms == MPR<double>::IntersectStatus::Intersect) { r.ok = 1; r.gjk_status = 10; finish(r, true); continue; }
        if (ms == MPR<double>::IntersectStatus::Separated) { r.ok = 0; r.gjk_status = 11; finish(r, true); continue; }
      }
      GJK<double> gjk(128, 1e-6);
      GJKSimplex<double> s;
      const GJK_Status gs = gjk.Evaluate(md, s, -Vec(1, 0, 0));
      r.gjk_status = (int)gs;
      if (!want_contact || gs != GJK_Status::Intersect) {
        r.ok = (!want_contact && gs == GJK_Status::Intersect) ? 1 : 0;
        finish(r, true);
        continue;
      }
      EPA<double> epa(256, 255, 1e-6);
      double depth = 0;
      Vec a, bb;
      const EPA_Status es = epa.Evaluate(s, md, &depth, &a, &bb);
      r.epa_status = (int)es;
      if (es != EPA_Status::Failed) {
        r.ok = 1;
        for (int k = 0; k < 3; ++k) { r.p0[k] = a[k]; r.p1[k] = bb[k]; }
        r.distance = -depth;
      }
      finish(r, true);
    }
  });
  return 0;
}

// The reference's MPR::RunDirectedPenetration (mpr.hpp:495-595) on every pair
// along dirs[i], 128 iterations, tolerance 1e-6: epa_status = its status,
// distance = distance_on_direction, p0 / p1 its witness points.
int ref_directed(const void* shapes, int n_shapes, const float* verts, const void* pairs, int n_pairs,
                 const float* dirs, RefResult* out, int n_threads) {
  const Prepared p = prepare((const ShapeRec*)shapes, n_shapes, verts);
  const PairRec* pr = (const PairRec*)pairs;
  parallelFor(n_pairs, n_threads, [&](int b, int e) {
    for (int i = b; i < e; ++i) {
      RefResult& r = out[i];
      r = RefResult{};
      const MinkowskiDiff<double> md = makeDiff(p, pr[i]);
      const Vec d(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]);
      typename MPR<double>::DirectedPenetrationData data;
      const auto st = MPR<double>::RunDirectedPenetration(md, d, data, 128, 1e-6);
      r.epa_status = (int)st;
      r.distance = data.distance_on_direction;
      for (int k = 0; k < 3; ++k) { r.p0[k] = data.p0_in_shape0_frame[k]; r.p1[k] = data.p1_in_shape0_frame[k]; }
      r.ok = st == MPR<double>::DirectedPenetrationStatus::OK ? 1 : 0;
    }
  });
  return 0;
}

// The reference's MPR::RunIncrementalMinimumPenetrationDistance
// (mpr_incremental_penetration.hpp:176-288) on every pair, with the
// fcl::collide settings (128 iterations, 1e-6, return on the first
// converged subroutine).
int ref_incremental(const void* shapes, int n_shapes, const float* verts, const void* pairs, int n_pairs,
                    const float* dirs, RefResult* out, int n_threads) {
  const Prepared p = prepare((const ShapeRec*)shapes, n_shapes, verts);
  const PairRec* pr = (const PairRec*)pairs;
  parallelFor(n_pairs, n_threads, [&](int b, int e) {
    for (int i = b; i < e; ++i) {
      RefResult& r = out[i];
      r = RefResult{};
      const MinkowskiDiff<double> md = makeDiff(p, pr[i]);
      const Vec d(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]);
      typename MPR<double>::IncrementalMinimumPenetrationData data{};
      const auto st = MPR<double>::RunIncrementalMinimumPenetrationDistance(md, d, data, 128, 1e-6, true);
      r.epa_status = (int)st;
      r.distance = data.minimum_penetration;
      for (int k = 0; k < 3; ++k) {
        r.normal[k] = data.penetration_direction[k];
        r.p0[k] = data.p0_in_shape0_frame[k];
        r.p1[k] = data.p1_in_shape0_frame[k];
      }
      r.ok = (st == MPR<double>::IncrementalPenetrationStatus::OK ||
              st == MPR<double>::IncrementalPenetrationStatus::IterationLimit) ? 1 : 0;
    }
  });
  return 0;
}

// The reference's MPR::Intersect with IntersectData (cvx_collide/mpr.hpp:
// 22-185) on the difference of shape a swept along disp[i] (unit axis in a's
// frame, distance; TranslationalCollisionGJK::setupMinkowskiDiff,
// narrowphase/detail/ccd/gjk_ccd-inl.h:7-18) and shape b: per pair 23
// doubles = status, count of set portal vertices, v0, v1, v2, v3, d1, d2, d3.
int ref_swept_portal(const void* shapes, int n_shapes, const float* verts, const void* pairs, int n_pairs,
                     const float* disp, int max_iter, double tol, double* out, int n_threads) {
  const Prepared p = prepare((const ShapeRec*)shapes, n_shapes, verts);
  const PairRec* pr = (const PairRec*)pairs;
  parallelFor(n_pairs, n_threads, [&](int b, int e) {
    for (int i = b; i < e; ++i) {
      MinkowskiDiff<double> md = makeDiff(p, pr[i]);
      GJKGeometryData<double> swept;
      swept.shape_type = GJKShapeType::ShapeSweptVolume;
      swept.vec3_data = Vec(disp[4 * (size_t)i], disp[4 * (size_t)i + 1], disp[4 * (size_t)i + 2]) *
                        (double)disp[4 * (size_t)i + 3];
      swept.user_ptr = &p.geo[pr[i].shape_a];
      md.shapes[0] = swept;
      MPR<double> mpr(max_iter, tol);
      MPR<double>::IntersectData data;
      const auto st = mpr.Intersect(md, &data);
      double* o = out + 23 * (size_t)i;
      for (int k = 0; k < 23; ++k) o[k] = std::numeric_limits<double>::quiet_NaN();
      o[0] = (double)(int)st;
      const Vec* vs[3] = {&data.v1, &data.v2, &data.v3};
      const Vec* ds[3] = {&data.v1_dir_in_support, &data.v2_dir_in_support, &data.v3_dir_in_support};
      int count = 0;
      while (count < 3 && !std::isnan((*vs[count])[0])) ++count;
      o[1] = count;
      for (int k = 0; k < 3; ++k) o[2 + k] = data.v0_interior[k];
      for (int j = 0; j < count; ++j)
        for (int k = 0; k < 3; ++k) {
          o[5 + 3 * j + k] = (*vs[j])[k];
          o[14 + 3 * j + k] = (*ds[j])[k];
        }
    }
  });
  return 0;
}

}  // extern "C"
