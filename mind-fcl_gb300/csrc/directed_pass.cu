// fcl::collide in the directed and the incremental penetration modes, one
// thread per pair: the boolean collide (closed-form solvers, else MPR with the
// GJK fallback), then MPR directed penetration along the pair's escape
// direction, or the incremental minimum-distance penetration from it as a
// hint (collisionPenetrationMPR, collision_penetration-inl.h:106-250; directed
// MPR mpr.hpp:495-701; incremental mpr_incremental_penetration.hpp:10-333).  Its own kernel so that the distance pass keeps its
// register allocation.
#include "analytic.cuh"
#include "gjk.cuh"
#include "kernels.h"
#include "mpr.cuh"

namespace fclg {

__global__ void __launch_bounds__(128, 4) directed_pass(BatchArgs b, QueryParams prm) {
  constexpr int LANES = 1;
  const Group<LANES> g = Group<LANES>::make();
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t pid = blockIdx.x * blockDim.x + threadIdx.x; pid < b.n_pairs; pid += stride) {
    const PairDev pr = load_pair(b.pairs, pid);
    if (pr.a >= b.n_shapes || pr.b >= b.n_shapes) {
      store_result(b.results, pid, -1.f, mk3(0, 0, 1), mk3(0, 0, 0), mk3(0, 0, 0), kGjkFailed, 0, false, false);
      continue;
    }
    MinkowskiSupport<LANES> sup;
    sup.A = load_shape(b.shapes, b.walk, pr.a);
    sup.B = load_shape(b.shapes, b.walk, pr.b);
    sup.pose = pr.pose;
    sup.verts = b.verts;
    sup.hull = b.hull;
    sup.g = g;
    // fcl::collide, useDirectedPenetration (collisionPenetrationMPR,
    // collision_penetration-inl.h:106-250): the boolean collide (closed
    // form for sphere pairs, else MPR with the GJK fallback), then MPR
    // directed penetration along the pair's escape direction (b.guess).
    bool hit;
    int32_t st;
    AnalyticContact ac;
    if (analytic_contact(sup.A, sup.B, pr.pose, ac)) {
      hit = ac.hit;
      st = (hit ? kGjkIntersect : kGjkSeparated) | kStatusAnalytic;
    } else {
      Mpr<MinkowskiSupport<LANES>> mpr{sup, prm.gjk_max_iter, prm.gjk_tol};
      const f3 v0 =
          load_interior(b.shapes, pr.a, sup.A.type) - pr.pose.apply(load_interior(b.shapes, pr.b, sup.B.type));
      const MprStatus ms = mpr.intersect(v0);
      if (ms != MprStatus::Failed) {
        hit = ms == MprStatus::Intersect;
        st = (hit ? kGjkIntersect : kGjkSeparated) | kStatusMpr;
      } else {
        Simplex s0;
        const GjkOut o = gjk_evaluate(sup, mk3(-1.f, 0.f, 0.f), prm.gjk_tol, prm.gjk_max_iter, false, s0);
        hit = o.status == kGjkIntersect;
        st = o.status;
      }
    }
    const f3 d = mk3(__ldg(b.guess + 3 * (size_t)pid), __ldg(b.guess + 3 * (size_t)pid + 1),
                     __ldg(b.guess + 3 * (size_t)pid + 2));
    float depth = -1.f;
    f3 p0 = mk3(0, 0, 0), p1 = mk3(0, 0, 0), n = d;
    int ds = -1;
    uint32_t iters = 0;
    bool ok = false;
    if (hit) {
      // computePenetrationMPR (collision_penetration-inl.h:106-184), 128 iterations
      Mpr<MinkowskiSupport<LANES>> mpr{sup, 128, prm.epa_tol};
      if (prm.incremental) {
        f3 dir;
        ds = mpr.incremental(d, depth, dir, p0, p1);
        ok = ds == 0 || ds == 4;  // at the iteration limit still a valid penetration
        if (ok) n = dir;
      } else {
        ds = mpr.directed(d, depth, p0, p1);
        ok = ds == 0;
      }
      iters = (uint32_t)mpr.iterations;
    }
    if (g.lane == 0) {
      st |= (prm.incremental ? kStatusIncremental : kStatusDirected) | ((ds + 1) << 8);
      store_result(b.results, pid, ok ? -depth : -1.f, n, p0, p1, st, iters, hit, ok);
    }
  }
}

cudaError_t launch_directed(const BatchArgs& b, const QueryParams& prm, int blocks, cudaStream_t st) {
  if (b.n_pairs == 0) return cudaSuccess;
  directed_pass<<<blocks, 128, 0, st>>>(b, prm);
  return cudaGetLastError();
}

}  // namespace fclg
