// ORACLE — test infrastructure only (see orc_convex.hpp).  C entry points over
// the FP64 restatement, taking the same packed shape / pair buffers that the
// GPU library takes, so tests can hand one set of numpy arrays to both.
//
// Threads: std::thread with static chunking of the pair list; every thread owns
// its solver objects, as the reference's re-entrant narrowphase allows
// (include/fcl/narrowphase/collision_interface-inl.h:18 builds a solver per call).
#include <chrono>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "orc_convex.hpp"

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

}  // extern "C"

namespace {

std::vector<orc::Shape> makeShapes(const ShapeRec* s, int n, const float* verts) {
  std::vector<orc::Shape> out((size_t)n);
  for (int i = 0; i < n; ++i) {
    orc::Shape& o = out[(size_t)i];
    o.type = s[i].type;
    for (int k = 0; k < 3; ++k) o.p[k] = (double)s[i].param[k];
    if (o.type == orc::kConvex) {
      o.verts = verts + 4 * (size_t)s[i].vert_offset;
      o.nv = (int)s[i].vert_count;
      o.interior = orc::convexMean(o.verts, o.nv);
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
int orc_collide(const void* shapes, int n_shapes, const float* verts, const void* pairs, int n_pairs,
                int want_contact, OrcResult* out, int n_threads) {
  if (n_pairs < 0 || n_shapes < 0) return -1;
  const auto sh = makeShapes((const ShapeRec*)shapes, n_shapes, verts);
  const PairRec* pr = (const PairRec*)pairs;
  const orc::SolverParams sp;
  parallelFor(n_pairs, n_threads, [&](int b, int e) {
    for (int i = b; i < e; ++i) {
      const orc::MinkDiff md = makeDiff(sh, pr[i]);
      fill(out[i], orc::intersect(md, sp, want_contact != 0, nullptr), true);
    }
  });
  return 0;
}

// Wall-clock seconds of orc_signed_distance over the pairs (for the CPU
// baseline; excludes nothing but the call itself).
double orc_time_signed_distance(const void* shapes, int n_shapes, const float* verts, const void* pairs, int n_pairs,
                                OrcResult* out, int n_threads) {
  const auto t0 = std::chrono::steady_clock::now();
  orc_signed_distance(shapes, n_shapes, verts, pairs, n_pairs, nullptr, out, n_threads, 0, 0, 0, 0, 0);
  const auto t1 = std::chrono::steady_clock::now();
  return std::chrono::duration<double>(t1 - t0).count();
}

}  // extern "C"
