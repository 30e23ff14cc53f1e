// ORACLE — test infrastructure only (see orc_convex.hpp).  C entry points over
// the FP64 restatement, taking the same packed shape / pair buffers that the
// GPU library takes, so tests can hand one set of numpy arrays to both.
//
// Threads: std::thread with static chunking of the pair list; every thread owns
// its solver objects, as the reference's re-entrant narrowphase allows
// (include/fcl/narrowphase/collision_interface-inl.h:18 builds a solver per call).
#include <chrono>
#include <cstdint>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "orc_analytic.hpp"
#include "orc_ccd.hpp"
#include "orc_convex.hpp"
#include "orc_mesh.hpp"
#include "orc_mesh_shape.hpp"

namespace {

struct ShapeRec {  // 32 bytes, same layout as fclg_shape
  int32_t type;
  uint32_t vert_offset;
  uint32_t vert_count;
  uint32_t reserved;
  float param[4];
};
struct PairRec {  // 64 bytes, same layout as fclg_pair
  uint32_t shape_a, shape_b;
  float rot[9];
  float trans[3];
  uint32_t flags, reserved;
};
static_assert(sizeof(ShapeRec) == 32, "shape layout");
static_assert(sizeof(PairRec) == 64, "pair layout");

}  // namespace

extern "C" {

struct OrcResult {
  double distance;
  double p0[3];
  double p1[3];
  double normal[3];
  int32_t ok;
  int32_t gjk_status;
  int32_t epa_status;
  int32_t gjk_iters;
  int32_t epa_iters;
  int32_t reserved;
};

int orc_result_size() { return (int)sizeof(OrcResult); }

// Convex walk tables for the next query calls over n_shapes shapes: off[i] =
// start of shape i's table in nbr (Convex::neighbors_ layout: nv row offsets,
// each row a count then vertex indices), -1 for a scan.  Null clears them.
void orc_set_walk(const int64_t* off, int n_shapes, const int32_t* nbr);

}  // extern "C"

namespace {

// Neighbour tables for the convex walk (orc_set_walk): per shape the offset of
// its table in g_walk_nbr, or -1.  Set before a query call, cleared after.
const int64_t* g_walk_off = nullptr;
const int32_t* g_walk_nbr = nullptr;
int g_walk_n = 0;

std::vector<orc::Shape> makeShapes(const ShapeRec* s, int n, const float* verts) {
  std::vector<orc::Shape> out((size_t)n);
  const bool walk = g_walk_off && g_walk_nbr && g_walk_n == n;
  for (int i = 0; i < n; ++i) {
    orc::Shape& o = out[(size_t)i];
    o.type = s[i].type;
    for (int k = 0; k < 3; ++k) o.p[k] = (double)s[i].param[k];
    if (o.type == orc::kConvex) {
      o.verts = verts + 4 * (size_t)s[i].vert_offset;
      o.nv = (int)s[i].vert_count;
      o.interior = orc::convexMean(o.verts, o.nv);
      if (walk && g_walk_off[i] >= 0) orc::initWalk(o, g_walk_nbr + g_walk_off[i]);
    }
  }
  return out;
}

orc::MinkDiff makeDiff(const std::vector<orc::Shape>& shapes, const PairRec& p) {
  orc::MinkDiff md;
  md.s0 = &shapes[p.shape_a];
  md.s1 = &shapes[p.shape_b];
  for (int k = 0; k < 9; ++k) md.to0.R[k] = (double)p.rot[k];
  md.to0.t = orc::V3(p.trans[0], p.trans[1], p.trans[2]);
  return md;
}

void fill(OrcResult& r, const orc::QueryOut& q, bool for_contact) {
  r.distance = q.distance;
  for (int k = 0; k < 3; ++k) { r.p0[k] = q.p0[k]; r.p1[k] = q.p1[k]; }
  orc::V3 n;
  if (q.ok && q.distance > 0 && !for_contact) {
    n = q.p1 - q.p0;  // separated: direction that moves shape b away
  } else {
    n = q.p0 - q.p1;  // penetrating: shape b escapes along +normal (gjk_solver-inl.h:117-121)
  }
  if (orc::sqn(n) <= 0) n = orc::V3(0, 0, 1);
  else orc::normalize(n);
  for (int k = 0; k < 3; ++k) r.normal[k] = n[k];
  r.ok = q.ok ? 1 : 0;
  r.gjk_status = q.gjk_status;
  r.epa_status = q.epa_status;
  r.gjk_iters = q.gjk_iters;
  r.epa_iters = q.epa_iters;
  r.reserved = 0;
}

template <typename F>
void parallelFor(int n, int n_threads, F&& f) {
  if (n_threads <= 1 || n < 2 * n_threads) {
    f(0, n);
    return;
  }
  std::vector<std::thread> th;
  const int chunk = (n + n_threads - 1) / n_threads;
  for (int t = 0; t < n_threads; ++t) {
    const int b = t * chunk, e = std::min(n, b + chunk);
    if (b >= e) break;
    th.emplace_back([&f, b, e] { f(b, e); });
  }
  for (auto& x : th) x.join();
}

orc::SolverParams params(int gjk_max_iter, double gjk_tol, int epa_max_faces, int epa_max_iter, double epa_tol) {
  orc::SolverParams sp;
  if (gjk_max_iter > 0) sp.gjk_max_iter = gjk_max_iter;
  if (gjk_tol > 0) sp.gjk_tol = gjk_tol;
  if (epa_max_faces > 0) sp.epa_max_faces = (size_t)epa_max_faces;
  if (epa_max_iter > 0) sp.epa_max_iter = epa_max_iter;
  if (epa_tol > 0) sp.epa_tol = epa_tol;
  return sp;
}

}  // namespace

extern "C" void orc_set_walk(const int64_t* off, int n_shapes, const int32_t* nbr) {
  g_walk_off = off;
  g_walk_nbr = nbr;
  g_walk_n = off ? n_shapes : 0;
}

extern "C" {

// GJKSolver<double>::shapeSignedDistance per pair (gjk_solver-inl.h:810-874):
// GJK separation distance for separated pairs, -EPA depth for overlapping ones.
// guess (nullable, float[n][3]) plays the role of GJKSolver::gjk_guess.
// Zero / negative solver parameters select the reference defaults.
int orc_signed_distance(const void* shapes, int n_shapes, const float* verts, const void* pairs, int n_pairs,
                        const float* guess, OrcResult* out, int n_threads, int gjk_max_iter, double gjk_tol,
                        int epa_max_faces, int epa_max_iter, double epa_tol) {
  if (n_pairs < 0 || n_shapes < 0) return -1;
  const auto sh = makeShapes((const ShapeRec*)shapes, n_shapes, verts);
  const PairRec* pr = (const PairRec*)pairs;
  const orc::SolverParams sp = params(gjk_max_iter, gjk_tol, epa_max_faces, epa_max_iter, epa_tol);
  parallelFor(n_pairs, n_threads, [&](int b, int e) {
    for (int i = b; i < e; ++i) {
      const orc::MinkDiff md = makeDiff(sh, pr[i]);
      orc::V3 g;
      const orc::V3* gp = nullptr;
      if (guess) { g = orc::V3(guess[3 * i], guess[3 * i + 1], guess[3 * i + 2]); gp = &g; }
      fill(out[i], orc::signedDistance(md, sp, gp), false);
    }
  });
  return 0;
}

// fcl::collide on a convex pair (gjk_solver-inl.h:70-137): want_contact = 0 is
// the boolean request (MPR, GJK fallback); 1 is useDefaultPenetration (GJK+EPA).
// fcl::collide on a shape pair (ShapeIntersectIndepImpl::run): the closed-form
// solvers for sphere pairs when use_analytic (gjk_solver-inl.h:209-218),
// otherwise MPR (boolean) or GJK + EPA (contact).  Analytic results carry
// gjk_status 20, the contact normal and pos +- depth / 2 along it as p0 / p1.
int orc_collide(const void* shapes, int n_shapes, const float* verts, const void* pairs, int n_pairs,
                int want_contact, int use_analytic, OrcResult* out, int n_threads) {
  if (n_pairs < 0 || n_shapes < 0) return -1;
  const auto sh = makeShapes((const ShapeRec*)shapes, n_shapes, verts);
  const PairRec* pr = (const PairRec*)pairs;
  const orc::SolverParams sp;
  parallelFor(n_pairs, n_threads, [&](int b, int e) {
    for (int i = b; i < e; ++i) {
      const orc::MinkDiff md = makeDiff(sh, pr[i]);
      orc::AContact ac;
      if (use_analytic && orc::analyticIntersect(*md.s0, *md.s1, md.to0, ac)) {
        orc::QueryOut q;
        q.ok = ac.hit;
        q.gjk_status = 20;
        q.distance = ac.hit ? -ac.depth : ac.separation;
        q.p0 = ac.pos + ac.normal * (0.5 * ac.depth);
        q.p1 = ac.pos - ac.normal * (0.5 * ac.depth);
        fill(out[i], q, true);
        if (ac.hit)
          for (int k = 0; k < 3; ++k) out[i].normal[k] = ac.normal[k];
        continue;
      }
      fill(out[i], orc::intersect(md, sp, want_contact != 0, nullptr), true);
    }
  });
  return 0;
}

// fcl::collide in the directed penetration mode (collisionPenetrationMPR,
// collision_penetration-inl.h:106-250): the boolean collide (closed-form
// sphere solvers, else MPR with the GJK fallback), then for colliding pairs
// MPR::DirectedPenetration along dirs[i] (shape b's escape direction in a's
// frame, unit).  Result: ok = collide; distance = -depth on direction (OK) or
// -1; p0 / p1 the witness points; normal = the direction; epa_status = the
// directed status (0 OK, 1 Failed, 2 FailedNoIntersect, 3 iteration limit).
int orc_collide_directed(const void* shapes, int n_shapes, const float* verts, const void* pairs, int n_pairs,
                         const float* dirs, OrcResult* out, int n_threads) {
  if (n_pairs < 0 || n_shapes < 0 || !dirs) return -1;
  const auto sh = makeShapes((const ShapeRec*)shapes, n_shapes, verts);
  const PairRec* pr = (const PairRec*)pairs;
  const orc::SolverParams sp;
  parallelFor(n_pairs, n_threads, [&](int b, int e) {
    for (int i = b; i < e; ++i) {
      const orc::MinkDiff md = makeDiff(sh, pr[i]);
      OrcResult& r = out[i];
      r = OrcResult{};
      orc::AContact ac;
      bool hit;
      if (orc::analyticIntersect(*md.s0, *md.s1, md.to0, ac)) hit = ac.hit;
      else hit = orc::intersect(md, sp, false, nullptr).ok;
      const orc::V3 d(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]);
      for (int k = 0; k < 3; ++k) r.normal[k] = d[k];
      r.ok = hit ? 1 : 0;
      r.distance = -1;
      r.epa_status = -1;
      if (!hit) continue;
      orc::MPR mpr(128, sp.epa_tol);
      orc::MPR::Directed pd;
      const int st = mpr.DirectedPenetration(md, d, pd);
      r.epa_status = st;
      if (st == 0) {
        r.distance = -pd.distance;
        for (int k = 0; k < 3; ++k) { r.p0[k] = pd.p0[k]; r.p1[k] = pd.p1[k]; }
      }
    }
  });
  return 0;
}

// The restated MPR::DirectedPenetration on every pair (no boolean gate), in
// the layout of ref_directed, for the bit-for-bit pin.
int orc_directed_raw(const void* shapes, int n_shapes, const float* verts, const void* pairs, int n_pairs,
                     const float* dirs, OrcResult* out, int n_threads) {
  if (n_pairs < 0 || n_shapes < 0 || !dirs) return -1;
  const auto sh = makeShapes((const ShapeRec*)shapes, n_shapes, verts);
  const PairRec* pr = (const PairRec*)pairs;
  parallelFor(n_pairs, n_threads, [&](int b, int e) {
    for (int i = b; i < e; ++i) {
      const orc::MinkDiff md = makeDiff(sh, pr[i]);
      OrcResult& r = out[i];
      r = OrcResult{};
      orc::MPR mpr(128, 1e-6);
      orc::MPR::Directed pd;
      const int st = mpr.DirectedPenetration(md, orc::V3(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]), pd);
      r.epa_status = st;
      r.distance = pd.distance;
      for (int k = 0; k < 3; ++k) { r.p0[k] = pd.p0[k]; r.p1[k] = pd.p1[k]; }
      r.ok = st == 0 ? 1 : 0;
    }
  });
  return 0;
}

// fcl::collide in the incremental minimum-distance penetration mode
// (computePenetrationMPR with is_incremental, collision_penetration-inl.h:
// 133-155): the boolean collide as in orc_collide_directed, then
// MPR::IncrementalMinimumPenetrationDistance from the hint dirs[i] for
// colliding pairs.  Result: ok = collide; distance = -depth and normal = the
// converged direction when the run is OK or at its iteration limit (both
// valid for the reference), else distance -1 and normal = the hint;
// epa_status = the incremental status (0 OK, 1 Failed, 2 FailedNoIntersect,
// 4 IterationLimit), -1 when not colliding.
int orc_collide_incremental(const void* shapes, int n_shapes, const float* verts, const void* pairs, int n_pairs,
                            const float* dirs, OrcResult* out, int n_threads) {
  if (n_pairs < 0 || n_shapes < 0 || !dirs) return -1;
  const auto sh = makeShapes((const ShapeRec*)shapes, n_shapes, verts);
  const PairRec* pr = (const PairRec*)pairs;
  const orc::SolverParams sp;
  parallelFor(n_pairs, n_threads, [&](int b, int e) {
    for (int i = b; i < e; ++i) {
      const orc::MinkDiff md = makeDiff(sh, pr[i]);
      OrcResult& r = out[i];
      r = OrcResult{};
      orc::AContact ac;
      bool hit;
      if (orc::analyticIntersect(*md.s0, *md.s1, md.to0, ac)) hit = ac.hit;
      else hit = orc::intersect(md, sp, false, nullptr).ok;
      const orc::V3 d(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]);
      for (int k = 0; k < 3; ++k) r.normal[k] = d[k];
      r.ok = hit ? 1 : 0;
      r.distance = -1;
      r.epa_status = -1;
      if (!hit) continue;
      orc::MPR mpr(128, sp.epa_tol);
      orc::MPR::Incremental pd;
      const int st = mpr.IncrementalPenetration(md, d, pd);
      r.epa_status = st;
      if (st == 0 || st == 4) {
        r.distance = -pd.depth;
        for (int k = 0; k < 3; ++k) { r.normal[k] = pd.dir[k]; r.p0[k] = pd.p0[k]; r.p1[k] = pd.p1[k]; }
      }
    }
  });
  return 0;
}

// The restated incremental penetration on every pair (no boolean gate), in
// the layout of ref_incremental, for the bit-for-bit pin: distance = depth.
int orc_incremental_raw(const void* shapes, int n_shapes, const float* verts, const void* pairs, int n_pairs,
                        const float* dirs, OrcResult* out, int n_threads) {
  if (n_pairs < 0 || n_shapes < 0 || !dirs) return -1;
  const auto sh = makeShapes((const ShapeRec*)shapes, n_shapes, verts);
  const PairRec* pr = (const PairRec*)pairs;
  parallelFor(n_pairs, n_threads, [&](int b, int e) {
    for (int i = b; i < e; ++i) {
      const orc::MinkDiff md = makeDiff(sh, pr[i]);
      OrcResult& r = out[i];
      r = OrcResult{};
      orc::MPR mpr(128, 1e-6);
      orc::MPR::Incremental pd;
      const int st = mpr.IncrementalPenetration(md, orc::V3(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]), pd);
      r.epa_status = st;
      r.distance = pd.depth;
      for (int k = 0; k < 3; ++k) { r.normal[k] = pd.dir[k]; r.p0[k] = pd.p0[k]; r.p1[k] = pd.p1[k]; }
      r.ok = (st == 0 || st == 4) ? 1 : 0;
    }
  });
  return 0;
}

// boxBox2 (box_box-inl.h:214-802) on two posed boxes in FP64, as
// boxBoxIntersect calls it (maxc 4): out = normal[3], depth, code, count, then
// count x (pos[3], depth).  Returns the contact count.
int orc_box_box(const double* side1, const double* R1, const double* T1, const double* side2, const double* R2,
                const double* T2, double* out) {
  orc::BoxContact c[4];
  orc::V3 normal;
  double depth = 0, sep = 0;
  int code = 0;
  const int n = orc::boxBox2(orc::V3(side1[0], side1[1], side1[2]), R1, orc::V3(T1[0], T1[1], T1[2]),
                             orc::V3(side2[0], side2[1], side2[2]), R2, orc::V3(T2[0], T2[1], T2[2]), normal, depth,
                             code, 4, c, sep);
  for (int k = 0; k < 3; ++k) out[k] = normal[k];
  out[3] = code ? depth : sep;
  out[4] = code;
  out[5] = n;
  for (int j = 0; j < n; ++j) {
    for (int k = 0; k < 3; ++k) out[6 + 4 * j + k] = c[j].pos[k];
    out[6 + 4 * j + 3] = c[j].depth;
  }
  return n;
}

// Support point of one shape for n directions (dirs, out: n x 3), through
// the same shape set-up (and walk tables) as the queries.
int orc_support(const void* shapes, int n_shapes, const float* verts, int shape, const double* dirs, int n,
                double* out) {
  if (shape < 0 || shape >= n_shapes) return -1;
  const auto sh = makeShapes((const ShapeRec*)shapes, n_shapes, verts);
  for (int i = 0; i < n; ++i) {
    const orc::V3 p = orc::support(sh[(size_t)shape], orc::V3(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]));
    for (int k = 0; k < 3; ++k) out[3 * i + k] = p[k];
  }
  return 0;
}

// Wall-clock seconds of the orc_signed_distance queries over the pairs (for
// the CPU baseline).  Shape set-up (vertex means, the walk's cached axis
// extremes) is outside the clock: fcl::Convex does it once at construction.
double orc_time_signed_distance(const void* shapes, int n_shapes, const float* verts, const void* pairs, int n_pairs,
                                OrcResult* out, int n_threads) {
  if (n_pairs < 0 || n_shapes < 0) return -1;
  const auto sh = makeShapes((const ShapeRec*)shapes, n_shapes, verts);
  const PairRec* pr = (const PairRec*)pairs;
  const orc::SolverParams sp = params(0, 0, 0, 0, 0);
  const auto t0 = std::chrono::steady_clock::now();
  parallelFor(n_pairs, n_threads, [&](int b, int e) {
    for (int i = b; i < e; ++i) fill(out[i], orc::signedDistance(makeDiff(sh, pr[i]), sp, nullptr), false);
  });
  const auto t1 = std::chrono::steady_clock::now();
  return std::chrono::duration<double>(t1 - t0).count();
}

// OrientedNodeBVHSolver::MeshIntersect with penetration off per pose
// (bvh_solver-inl.h:74-164): b posed by poses[i] (12 floats, rotation
// row-major then translation) in a's frame, traversing the given flattened
// OBB trees; up to max_contacts (a, b) triangle pairs per pose in the
// reference's traversal order.  max_contacts = 0 means no limit (every
// colliding pair; pairs must then hold pair_cap entries per pose).
int orc_mesh_collide(const void* nodes_a, const float* tris_a, const void* nodes_b, const float* tris_b,
                     const float* poses, int n_poses, int max_contacts, int pair_cap, uint8_t* flags, uint32_t* counts,
                     int32_t* pairs, int n_threads) {
  const orc::MeshNode* na = (const orc::MeshNode*)nodes_a;
  const orc::MeshNode* nb = (const orc::MeshNode*)nodes_b;
  parallelFor(n_poses, n_threads, [&](int b, int e) {
    std::vector<std::pair<int, int>> c;
    for (int i = b; i < e; ++i) {
      orc::Mat3 R;
      for (int k = 0; k < 9; ++k) R.m[k] = poses[12 * (size_t)i + k];
      const double T[3] = {poses[12 * (size_t)i + 9], poses[12 * (size_t)i + 10], poses[12 * (size_t)i + 11]};
      orc::meshIntersect(na, tris_a, nb, tris_b, R, T, max_contacts > 0 ? (size_t)max_contacts : SIZE_MAX, c);
      flags[i] = c.empty() ? 0 : 1;
      counts[i] = (uint32_t)c.size();
      const size_t cap = (size_t)pair_cap;
      for (size_t k = 0; k < c.size() && k < cap; ++k) {
        pairs[2 * (cap * i + k)] = c[k].first;
        pairs[2 * (cap * i + k) + 1] = c[k].second;
      }
    }
  });
  return 0;
}

// fcl::collide(mesh, shape) with penetration off per query: shape shape_ids[i]
// posed by poses[i] (12 floats: rotation row-major, translation) in the mesh
// frame (MeshShapeIntersect, bvh_solver-inl.h:6-72).  max_contacts 0: every
// colliding triangle.  Writes flags, counts and up to pair_cap triangle ids
// per query.
int orc_mesh_shape_collide(const void* nodes, const float* tris, const void* shapes, int n_shapes,
                           const float* verts, const uint32_t* shape_ids, const float* poses, int n, int max_contacts,
                           int pair_cap, uint8_t* flags, uint32_t* counts, int32_t* tri_ids, int n_threads) {
  const orc::MeshNode* nd = (const orc::MeshNode*)nodes;
  const auto sh = makeShapes((const ShapeRec*)shapes, n_shapes, verts);
  const orc::SolverParams sp;
  parallelFor(n, n_threads, [&](int b, int e) {
    std::vector<int> c;
    for (int i = b; i < e; ++i) {
      orc::Iso X;
      for (int k = 0; k < 9; ++k) X.R[k] = poses[12 * (size_t)i + k];
      X.t = orc::V3(poses[12 * (size_t)i + 9], poses[12 * (size_t)i + 10], poses[12 * (size_t)i + 11]);
      const uint32_t si = shape_ids[i];
      c.clear();
      if (si < (uint32_t)n_shapes)
        orc::meshShapeIntersect(nd, tris, sh[si], X, max_contacts > 0 ? (size_t)max_contacts : SIZE_MAX, sp, c);
      flags[i] = c.empty() ? 0 : 1;
      counts[i] = (uint32_t)c.size();
      for (size_t k = 0; k < c.size() && k < (size_t)pair_cap; ++k) tri_ids[(size_t)pair_cap * i + k] = c[k];
    }
  });
  return 0;
}

// Mesh-shape collide with penetration on: per query up to max_contacts
// contacts (pair_cap slots per query): tri_ids, contacts[8] = pos, normal,
// depth, EPA status (-1 for the closed-form sphere).
int orc_mesh_shape_contacts(const void* nodes, const float* tris, const void* shapes, int n_shapes,
                            const float* verts, const uint32_t* shape_ids, const float* poses, int n, int max_contacts,
                            int pair_cap, uint32_t* counts, int32_t* tri_ids, double* contacts, int n_threads) {
  const orc::MeshNode* nd = (const orc::MeshNode*)nodes;
  const auto sh = makeShapes((const ShapeRec*)shapes, n_shapes, verts);
  const orc::SolverParams sp;
  parallelFor(n, n_threads, [&](int b, int e) {
    std::vector<orc::MsContact> c;
    for (int i = b; i < e; ++i) {
      orc::Iso X;
      for (int k = 0; k < 9; ++k) X.R[k] = poses[12 * (size_t)i + k];
      X.t = orc::V3(poses[12 * (size_t)i + 9], poses[12 * (size_t)i + 10], poses[12 * (size_t)i + 11]);
      const uint32_t si = shape_ids[i];
      c.clear();
      if (si < (uint32_t)n_shapes)
        orc::meshShapeContacts(nd, tris, sh[si], X, max_contacts > 0 ? (size_t)max_contacts : SIZE_MAX, sp, c);
      counts[i] = (uint32_t)c.size();
      for (size_t k = 0; k < c.size() && k < (size_t)pair_cap; ++k) {
        tri_ids[(size_t)pair_cap * i + k] = c[k].tri;
        double* o = contacts + 8 * ((size_t)pair_cap * i + k);
        for (int j = 0; j < 3; ++j) { o[j] = c[k].pos[j]; o[3 + j] = c[k].normal[j]; }
        o[6] = c[k].depth;
        o[7] = c[k].epa_status;
      }
    }
  });
  return 0;
}

// CollisionObject::computeAABB (narrowphase/collision_object-inl.h:141-154)
// of object i = shape ids[i] posed by poses[i] (12 floats, world), in FP64:
// out[6 i ..] = lo, hi.  The local box is computeBV<AABB>(shape, identity)
// (geometry/shape/utility-inl.h:70-219, 770-776; a hull's from its vertices,
// convex-inl.h:76-87), its centre and half-diagonal radius as
// computeLocalAABB stores them (box-inl.h:74-80).
int orc_object_aabbs(const void* shapes, int n_shapes, const float* verts, const uint32_t* ids, const float* poses,
                     int n, double* out) {
  const ShapeRec* sr = (const ShapeRec*)shapes;
  for (int i = 0; i < n; ++i) {
    const uint32_t s = ids[i];
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    if (s < (uint32_t)n_shapes) {
      const ShapeRec& r = sr[s];
      const double p0 = r.param[0], p1 = r.param[1], p2 = r.param[2];
      switch (r.type) {
        case orc::kBox: hi[0] = 0.5 * p0; hi[1] = 0.5 * p1; hi[2] = 0.5 * p2; break;
        case orc::kSphere: hi[0] = hi[1] = hi[2] = p0; break;
        case orc::kCapsule: hi[0] = hi[1] = p0; hi[2] = 0.5 * p1 + p0; break;
        case orc::kCylinder: hi[0] = hi[1] = p0; hi[2] = 0.5 * p1; break;
        default: {
          for (int k = 0; k < 3; ++k) { lo[k] = 1e300; hi[k] = -1e300; }
          for (uint32_t v = 0; v < r.vert_count; ++v)
            for (int k = 0; k < 3; ++k) {
              const double x = verts[4 * ((size_t)r.vert_offset + v) + k];
              lo[k] = std::min(lo[k], x);
              hi[k] = std::max(hi[k], x);
            }
        }
      }
      if (r.type != orc::kConvex)
        for (int k = 0; k < 3; ++k) lo[k] = -hi[k];
    } else {
      for (int k = 0; k < 3; ++k) { lo[k] = 1e300; hi[k] = -1e300; }
      for (int k = 0; k < 3; ++k) { out[6 * i + k] = lo[k]; out[6 * i + 3 + k] = hi[k]; }
      continue;
    }
    const float* P = poses + 12 * (size_t)i;
    bool identity = true;
    for (int k = 0; k < 9; ++k) identity = identity && std::abs((double)P[k] - ((k % 4 == 0) ? 1.0 : 0.0)) <= 1e-12;
    const double t[3] = {P[9], P[10], P[11]};
    if (identity) {
      for (int k = 0; k < 3; ++k) { out[6 * i + k] = lo[k] + t[k]; out[6 * i + 3 + k] = hi[k] + t[k]; }
      continue;
    }
    const double c[3] = {0.5 * (lo[0] + hi[0]), 0.5 * (lo[1] + hi[1]), 0.5 * (lo[2] + hi[2])};
    const double d[3] = {lo[0] - c[0], lo[1] - c[1], lo[2] - c[2]};
    const double rad = std::sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]);
    for (int k = 0; k < 3; ++k) {
      const double cw = (((double)P[3 * k] * c[0] + (double)P[3 * k + 1] * c[1]) + (double)P[3 * k + 2] * c[2]) + t[k];
      out[6 * i + k] = cw - rad;
      out[6 * i + 3 + k] = cw + rad;
    }
  }
  return 0;
}

// Every pair (i < j) of boxes (6 values each, lo then hi) that overlap as
// AABB::overlap decides (apart only if one starts past the other's end), by
// brute force; returns the count, writes up to cap pairs.
int orc_aabb_pairs(const double* box, int n, uint32_t* pairs, int cap) {
  int m = 0;
  for (int i = 0; i < n; ++i)
    for (int j = i + 1; j < n; ++j) {
      const double* a = box + 6 * (size_t)i;
      const double* b = box + 6 * (size_t)j;
      bool apart = false;
      for (int k = 0; k < 3; ++k) apart = apart || a[k] > b[3 + k] || b[k] > a[3 + k];
      if (apart) continue;
      if (m < cap) { pairs[2 * m] = (uint32_t)i; pairs[2 * m + 1] = (uint32_t)j; }
      ++m;
    }
  return m;
}

// The same pair set by sorting on the lower x bound and sweeping (the CPU
// baseline of the broadphase; the reference walks a binary AABB tree, also
// O(n log n + pairs)).
int orc_sweep_pairs(const double* box, int n, uint32_t* pairs, int cap) {
  std::vector<int> order((size_t)n);
  for (int i = 0; i < n; ++i) order[(size_t)i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return box[6 * (size_t)a] < box[6 * (size_t)b]; });
  int m = 0;
  for (int k = 0; k < n; ++k) {
    const double* a = box + 6 * (size_t)order[(size_t)k];
    for (int q = k + 1; q < n; ++q) {
      const double* b = box + 6 * (size_t)order[(size_t)q];
      if (b[0] > a[3]) break;
      if (a[1] > b[4] || b[1] > a[4] || a[2] > b[5] || b[2] > a[5]) continue;
      if (m < cap) {
        const uint32_t i = (uint32_t)order[(size_t)k], j = (uint32_t)order[(size_t)q];
        pairs[2 * m] = std::min(i, j);
        pairs[2 * m + 1] = std::max(i, j);
      }
      ++m;
    }
  }
  return m;
}

// Every colliding triangle of one query by brute force over all triangles.
int orc_mesh_shape_all(const float* tris, int n_tris, const void* shapes, int n_shapes, const float* verts,
                       uint32_t shape_id, const float* pose, int32_t* tri_ids, int cap) {
  const auto sh = makeShapes((const ShapeRec*)shapes, n_shapes, verts);
  const orc::SolverParams sp;
  orc::Iso X;
  for (int k = 0; k < 9; ++k) X.R[k] = pose[k];
  X.t = orc::V3(pose[9], pose[10], pose[11]);
  int cnt = 0;
  for (int t = 0; t < n_tris; ++t)
    if (orc::shapeTriangleIntersect(sh[shape_id], X, tris + 12 * (size_t)t, sp)) {
      if (cnt < cap) tri_ids[cnt] = t;
      ++cnt;
    }
  return cnt;
}

// Every colliding triangle pair of one pose by brute force (returns the count;
// writes up to cap pairs).
int orc_mesh_allpairs(const float* tris_a, int n_a, const float* tris_b, int n_b, const float* pose, int32_t* pairs,
                      int cap) {
  orc::Mat3 R;
  for (int k = 0; k < 9; ++k) R.m[k] = pose[k];
  const double T[3] = {pose[9], pose[10], pose[11]};
  std::vector<std::pair<int, int>> c;
  orc::allPairs(tris_a, n_a, tris_b, n_b, R, T, c);
  for (size_t k = 0; k < c.size() && (int)k < cap; ++k) {
    pairs[2 * k] = c[k].first;
    pairs[2 * k + 1] = c[k].second;
  }
  return (int)c.size();
}

// The reference's OBBRSS tree over nt triangles (FP64 vertices, restated
// BVHModel<OBBRSS<double>>::endModel).  Returns the node count (2 nt - 1);
// f64 (may be null): per node axis (9, row-major), To, extent, size; i32 (may
// be null): first_child, first_primitive, num_primitives; prim (may be null):
// the primitive order after the build.
int orc_ref_tree(const double* V, const int32_t* T, int nt, double* f64, int32_t* i32, uint32_t* prim) {
  std::vector<orc::RefNode> nodes;
  std::vector<uint32_t> pr;
  orc::buildRefTree(V, T, nt, nodes, pr);
  for (size_t i = 0; i < nodes.size(); ++i) {
    const orc::RefNode& n = nodes[i];
    if (f64) {
      double* d = f64 + 16 * i;
      for (int k = 0; k < 9; ++k) d[k] = n.axis[k];
      for (int k = 0; k < 3; ++k) {
        d[9 + k] = n.To[k];
        d[12 + k] = n.extent[k];
      }
      d[15] = n.size;
    }
    if (i32) {
      i32[3 * i] = n.first_child;
      i32[3 * i + 1] = n.first_primitive;
      i32[3 * i + 2] = n.num_primitives;
    }
  }
  if (prim)
    for (int i = 0; i < nt; ++i) prim[i] = pr[i];
  return (int)nodes.size();
}

// MeshIntersect per pose over the reference's own trees, rebuilt here from the
// FP64 vertices (restated endModel): mesh a at the identity, mesh b posed by
// poses[i] (12 doubles: rotation row-major, translation).  counts[i] = the
// number of contacts (at most max_contacts), pairs[i][k] = (b1, b2) of contact
// k in the reference's order, for k < stride.
int orc_ref_mesh_collide(const double* Va, const int32_t* Ta, int nta, const double* Vb, const int32_t* Tb, int ntb,
                         const double* poses, int n_poses, int max_contacts, int32_t* counts, int32_t* pairs,
                         int stride, int n_threads) {
  if (nta <= 0 || ntb <= 0 || max_contacts <= 0) return -1;
  std::vector<orc::RefNode> na, nb;
  std::vector<uint32_t> pa, pb;
  orc::buildRefTree(Va, Ta, nta, na, pa);
  orc::buildRefTree(Vb, Tb, ntb, nb, pb);
  parallelFor(n_poses, n_threads, [&](int b, int e) {
    std::vector<std::pair<int, int>> c;
    for (int i = b; i < e; ++i) {
      orc::Mat3 R;
      for (int k = 0; k < 9; ++k) R.m[k] = poses[12 * (size_t)i + k];
      const double T[3] = {poses[12 * (size_t)i + 9], poses[12 * (size_t)i + 10], poses[12 * (size_t)i + 11]};
      orc::meshIntersectRef(na.data(), Va, Ta, nb.data(), Vb, Tb, R, T, (size_t)max_contacts, c);
      counts[i] = (int32_t)c.size();
      for (size_t k = 0; k < c.size() && (int)k < stride; ++k) {
        pairs[2 * ((size_t)stride * i + k)] = c[k].first;
        pairs[2 * ((size_t)stride * i + k) + 1] = c[k].second;
      }
    }
  });
  return 0;
}

// One triangle-triangle verdict (intersect_Triangle, boolean).
int orc_tri_tri(const double* p /* 9 */, const double* q /* 9 */, const double* pose /* 12 */) {
  orc::Mat3 R;
  for (int k = 0; k < 9; ++k) R.m[k] = pose[k];
  const double T[3] = {pose[9], pose[10], pose[11]};
  return orc::intersectTriangle({p[0], p[1], p[2]}, {p[3], p[4], p[5]}, {p[6], p[7], p[8]}, {q[0], q[1], q[2]},
                                {q[3], q[4], q[5]}, {q[6], q[7], q[8]}, R, T)
             ? 1
             : 0;
}

// ------------------------------------------------------ translational CCD --
// Per pair: shape a moving along disp[i] = (unit axis in a's frame, distance)
// against shape b at the pair's pose (fcl::translational_ccd).
struct OrcCcd {
  int32_t collide, mpr_status, box_tested, reserved;
  double toc_lo, toc_hi;
};
static_assert(sizeof(OrcCcd) == 32, "ccd layout");

int orc_translational_ccd(const void* shapes, int n_shapes, const float* verts, const void* pairs, int n_pairs,
                          const float* disp, int toc_type, double zero_tol, int max_iter, double tol, OrcCcd* out,
                          int n_threads) {
  if (n_pairs < 0 || n_shapes < 0 || !disp || toc_type < 0 || toc_type > 2) return -1;
  const auto sh = makeShapes((const ShapeRec*)shapes, n_shapes, verts);
  const PairRec* pr = (const PairRec*)pairs;
  parallelFor(n_pairs, n_threads, [&](int b, int e) {
    for (int i = b; i < e; ++i) {
      const orc::MinkDiff md = makeDiff(sh, pr[i]);
      const orc::V3 axis(disp[4 * (size_t)i], disp[4 * (size_t)i + 1], disp[4 * (size_t)i + 2]);
      const orc::CcdOut o = orc::translationalCcd(*md.s0, *md.s1, md.to0, axis, disp[4 * (size_t)i + 3],
                                                  (orc::TocRequest)toc_type, zero_tol, max_iter, tol);
      out[i] = OrcCcd{o.collide ? 1 : 0, o.mpr_status, o.box_tested ? 1 : 0, 0, o.toc.lo, o.toc.hi};
    }
  });
  return 0;
}

// MPR::Intersect on the swept-volume difference with its IntersectData, in
// the layout of ref_swept_portal for the bit-for-bit pin: per pair 23
// doubles = status, count, v0, v1, v2, v3, d1, d2, d3 (unset entries NaN).
int orc_swept_portal(const void* shapes, int n_shapes, const float* verts, const void* pairs, int n_pairs,
                     const float* disp, int max_iter, double tol, double* out, int n_threads) {
  if (n_pairs < 0 || n_shapes < 0 || !disp) return -1;
  const auto sh = makeShapes((const ShapeRec*)shapes, n_shapes, verts);
  const PairRec* pr = (const PairRec*)pairs;
  parallelFor(n_pairs, n_threads, [&](int b, int e) {
    for (int i = b; i < e; ++i) {
      orc::MinkDiff md = makeDiff(sh, pr[i]);
      const orc::V3 axis(disp[4 * (size_t)i], disp[4 * (size_t)i + 1], disp[4 * (size_t)i + 2]);
      md.swept = true;
      md.sweep = axis * (double)disp[4 * (size_t)i + 3];
      orc::MPR mpr(max_iter, tol);
      orc::MPRPortal P;
      const orc::MPRStatus st = mpr.Intersect(md, &P);
      double* o = out + 23 * (size_t)i;
      for (int k = 0; k < 23; ++k) o[k] = std::numeric_limits<double>::quiet_NaN();
      o[0] = (double)(int)st;
      o[1] = P.count;
      for (int k = 0; k < 3; ++k) o[2 + k] = P.v0[k];
      for (int j = 0; j < P.count; ++j)
        for (int k = 0; k < 3; ++k) {
          o[5 + 3 * j + k] = P.v[j][k];
          o[14 + 3 * j + k] = P.d[j][k];
        }
    }
  });
  return 0;
}

// The box pieces alone, for the reference's interval tests
// (test/ccd/test_box_pair_ccd.cpp): one axis (scalar, signed displacement,
// unscaled interval), three axes (scaled), and a box pair.  Each returns
// 1 when empty / disjoint and writes the interval to lo_hi.
int orc_box_axis(double h1, double d, double h2, double off, double* lo_hi) {
  orc::Interval t;
  const bool e = orc::boxAxisEmptySigned(h1, d, h2, off, t);
  lo_hi[0] = t.lo;
  lo_hi[1] = t.hi;
  return e ? 1 : 0;
}

int orc_box_axes3(const double* h1, const double* d, const double* h2, const double* off, double zero_tol,
                  double* lo_hi) {
  orc::Interval t;
  const bool e = orc::boxAxes3Empty(h1, d, h2, off, t, zero_tol);
  lo_hi[0] = t.lo;
  lo_hi[1] = t.hi;
  return e ? 1 : 0;
}

int orc_box_pair_ccd(const double* h1, const double* axis, double dist, const double* R, const double* t,
                     const double* h2, double zero_tol, double* lo_hi) {
  orc::Interval iv;
  const bool e = orc::boxPairDisjoint(h1, orc::V3(axis[0], axis[1], axis[2]), dist, R, orc::V3(t[0], t[1], t[2]), h2,
                                      zero_tol, iv);
  lo_hi[0] = iv.lo;
  lo_hi[1] = iv.hi;
  return e ? 1 : 0;
}

}  // extern "C"
