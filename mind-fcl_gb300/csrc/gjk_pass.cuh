// GJK pass of a convex query batch (kernel template; instantiated two lane
// counts per translation unit, gjk_pass_l*.cu, so the units compile in
// parallel): one group of LANES lanes per pair, GJK
// boolean (or MPR for a boolean fcl::collide) and, for separated pairs, the GJK
// separation distance; overlapping pairs are appended (warp-aggregated
// atomics) to a compact work list with their final simplex for the EPA pass
// (epa_pass.cu).  The two passes are stream-ordered with no host round trip
// between them: the EPA grid reads the list length from device memory, so a
// query can be captured into a CUDA graph.
#pragma once
#include "analytic.cuh"
#include "gjk.cuh"
#include "kernels.h"
#include "mpr.cuh"

namespace fclg {

namespace {

__device__ __forceinline__ void write_simplex(float4* __restrict__ rec, uint32_t slot, const Simplex& s, int iters) {
  float f[28];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    f[1 + 6 * i + 0] = s.a[i].x;
    f[1 + 6 * i + 1] = s.a[i].y;
    f[1 + 6 * i + 2] = s.a[i].z;
    f[1 + 6 * i + 3] = s.b[i].x;
    f[1 + 6 * i + 4] = s.b[i].y;
    f[1 + 6 * i + 5] = s.b[i].z;
  }
  f[0] = __int_as_float(s.rank);
  f[25] = __int_as_float(iters);
  f[26] = 0.f;
  f[27] = 0.f;
  float4* r = rec + 7 * (size_t)slot;
#pragma unroll
  for (int k = 0; k < 7; ++k) r[k] = make_float4(f[4 * k], f[4 * k + 1], f[4 * k + 2], f[4 * k + 3]);
}

__device__ __forceinline__ uint32_t aggregated_slot(uint32_t* counter) {
  const unsigned m = __activemask();
  const unsigned lane = threadIdx.x & 31u;
  const int leader = __ffs(m) - 1;
  uint32_t base = 0;
  if ((int)lane == leader) base = atomicAdd(counter, (uint32_t)__popc(m));
  base = __shfl_sync(m, base, leader);
  return base + (uint32_t)__popc(m & ((1u << lane) - 1u));
}

__device__ __forceinline__ void store_invalid(float4* out, uint32_t pid) {
  store_result(out, pid, -1.f, mk3(0, 0, 1), mk3(0, 0, 0), mk3(0, 0, 0), kGjkFailed, 0, false, false);
}

}  // namespace

// A run from the learned direction stands for a separation certificate (with
// certified points when distances are wanted) or for an overlap that needs no
// EPA.
__device__ __forceinline__ bool warm_keep(const GjkOut& o, const QueryParams& prm) {
  return (o.status == kGjkSeparated && (o.point_valid || !prm.want_distance)) ||
         (o.status == kGjkIntersect && !prm.want_epa);
}

// A separated run under the certified stop that ended without a certified
// distance (no progress before the certificate, or the iteration limit).
__device__ __forceinline__ bool uncertified(const GjkOut& o, const QueryParams& prm) {
  return o.status == kGjkSeparated && prm.want_distance && !o.point_valid;
}

// The tail of a pair once its GJK run is over: the EPA hand-off for an
// overlapping pair, else the result record (shared by both GJK kernels).
__device__ __forceinline__ void finish_pair(const BatchArgs& b, const QueryParams& prm, const EpaQueue& q,
                                            uint32_t pid, const GjkOut& o, const Simplex& s) {
  if (o.status == kGjkIntersect) {
    if (prm.want_epa) {
      const uint32_t slot = aggregated_slot(q.count);
      q.list[slot] = pid;
      write_simplex(q.rec, slot, s, o.iterations);
      return;
    }
    store_result(b.results, pid, 0.f, mk3(0, 0, 1), mk3(0, 0, 0), mk3(0, 0, 0), kGjkIntersect,
                 (uint32_t)o.iterations, true, true);
    return;
  }
  if (!prm.want_distance) {
    store_result(b.results, pid, 0.f, mk3(0, 0, 1), mk3(0, 0, 0), mk3(0, 0, 0), o.status, (uint32_t)o.iterations,
                 false, o.status == kGjkSeparated);
    return;
  }
  // shapeSignedDistance: valid only for a separation certificate with valid points
  const bool ok = (o.status == kGjkSeparated) && o.point_valid;
  const f3 dv = o.p1 - o.p0;
  const float dist = ok ? nrm(dv) : -1.f;
  f3 nrmv = normalized(dv);
  if (!(sqn(nrmv) > 0.f)) nrmv = mk3(0, 0, 1);
  store_result(b.results, pid, dist, nrmv, o.p0, o.p1, o.status, (uint32_t)o.iterations, false, ok);
}

// CTAs per SM the GJK passes are compiled for (96 registers, a few spilled):
// five beat four at 128 registers (mixed 1.75 -> 1.68 ms, arm 35.4 -> 32.7 ms).
#ifndef FCLG_GJK_MINB
#define FCLG_GJK_MINB 5
#endif
// Kernel variants: PLAIN compiles the GJK run from the plain direction only
// (queries without closed-form pairs, MPR or a learned start: the distance
// entry points), which keeps the kernel's code small enough for the
// instruction cache; FULL compiles every path and selects by prm / b.guess.
// Both give the same results on the queries PLAIN serves.
// SPLIT is PLAIN's boolean phase alone: a separated pair goes to the
// DistList for gjk_dist_pass (distance queries only).  SPLIT_WARM is the
// boolean phase of FULL's learned-start runs (the learned direction, then the
// plain one for a pair it does not separate), handing separated pairs over
// the same way.
enum : int { kPassPlain = 0, kPassFull = 1, kPassSplit = 2, kPassSplitWarm = 3 };
// DistList record stages
enum : int { kStagePlain = 0, kStageLearned = 1, kStagePlainCertified = 2 };

__device__ __forceinline__ void push_dist(const DistList& dl, uint32_t pid, const Simplex& s, int before,
                                          int bool_iters, int stage) {
  const uint32_t r = aggregated_slot(dl.count);
  float4* o = dl.rec + 3 * (size_t)r;
  o[0] = make_float4(__uint_as_float(pid), __int_as_float(before), __int_as_float(bool_iters), __int_as_float(stage));
  o[1] = make_float4(s.a[0].x, s.a[0].y, s.a[0].z, s.b[0].x);
  o[2] = make_float4(s.b[0].y, s.b[0].z, 0.f, 0.f);
}
#ifndef FCLG_GJK_PLAIN_VARIANT
#define FCLG_GJK_PLAIN_VARIANT 1
#endif

template <int LANES, int MODE>
__global__ void __launch_bounds__(128, FCLG_GJK_MINB) gjk_pass(BatchArgs b, QueryParams prm, EpaQueue q,
                                                   const uint32_t* __restrict__ order,
                                                   const uint32_t* __restrict__ range, uint32_t* next,
                                                   DistList dl) {
  uint32_t begin = 0, end = b.n_pairs;
  if (range) {
    begin = range[0];
    end = range[1];
  }
  const Group<LANES> g = Group<LANES>::make();
  // A warp runs 32 / LANES pairs at a time.  With a counter (next, zero
  // before the launch) it takes its next pairs there as it finishes a round,
  // so a persistent grid's warps end together; without one, warp w takes
  // rounds w, w + W, ... (W warps in the grid).
  constexpr uint32_t kPer = 32 / LANES;
  const uint32_t slot = (threadIdx.x & 31u) / LANES;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t n_warps = (gridDim.x * blockDim.x) >> 5;
  auto take = [&](uint32_t done) -> uint32_t {
    if (!next) return done + n_warps * kPer;
    uint32_t k = 0;
    if ((threadIdx.x & 31u) == 0) k = atomicAdd(next, kPer);
    return __shfl_sync(0xFFFFFFFFu, k, 0);
  };
  const uint32_t n_items = end > begin ? end - begin : 0u;
  for (uint32_t round = next ? take(0) : warp * kPer; round < n_items; round = take(round)) {
    const uint32_t item = begin + round + slot;
    if (item >= end) continue;
    const uint32_t pid = order ? order[item] : item;
    const PairDev pr = load_pair(b.pairs, pid);
    if (pr.a >= b.n_shapes || pr.b >= b.n_shapes) {
      if (g.lane == 0) store_invalid(b.results, pid);
      continue;
    }
    MinkowskiSupport<LANES> sup;
    sup.A = load_shape(b.shapes, LANES == 1 ? b.walk : nullptr, pr.a);
    sup.B = load_shape(b.shapes, LANES == 1 ? b.walk : nullptr, pr.b);
    sup.pose = pr.pose;
    sup.verts = b.verts;
    sup.hull = b.hull;
    sup.g = g;
    // GJKSolver's default guess (1, 0, 0), gjk_solver-inl.h:1129
    const f3 plain = mk3(1.f, 0.f, 0.f);
    if (MODE == kPassFull && prm.analytic) {
      // fcl::collide: closed-form solvers for sphere pairs (gjk_solver-inl.h:209-218)
      AnalyticContact ac;
      if (analytic_contact(sup.A, sup.B, pr.pose, ac)) {
        if (g.lane == 0) {
          const int32_t st = (ac.hit ? kGjkIntersect : kGjkSeparated) | kStatusAnalytic;
          if (ac.hit) {
            const f3 half = ac.normal * (0.5f * ac.depth);
            store_result(b.results, pid, -ac.depth, ac.normal, ac.pos + half, ac.pos - half, st, 0u, true, true);
          } else {
            store_result(b.results, pid, ac.separation, ac.normal, mk3(0, 0, 0), mk3(0, 0, 0), st, 0u, false,
                         prm.want_distance != 0);
          }
        }
        continue;
      }
    }
    int mpr_iters = 0;
    if (MODE == kPassFull && prm.use_mpr) {
      // fcl::collide without contact: MPR decides, GJK only when MPR fails
      // (ShapeIntersectIndepImpl::run, gjk_solver-inl.h:86-97)
      Mpr<MinkowskiSupport<LANES>> mpr{sup, prm.gjk_max_iter, prm.gjk_tol};
      const f3 v0 = load_interior(b.shapes, pr.a, sup.A.type) - pr.pose.apply(load_interior(b.shapes, pr.b, sup.B.type));
      const MprStatus ms = mpr.intersect(v0);
      mpr_iters = mpr.iterations;
      if (ms != MprStatus::Failed) {
        if (g.lane == 0) {
          const bool hit = ms == MprStatus::Intersect;
          store_result(b.results, pid, 0.f, mk3(0, 0, 1), mk3(0, 0, 0), mk3(0, 0, 0),
                       (hit ? kGjkIntersect : kGjkSeparated) | kStatusMpr, (uint32_t)mpr_iters, hit, hit);
        }
        continue;
      }
    }
    Simplex s;
    GjkOut o;
    if (MODE == kPassSplit) {
      // gjk_evaluate's boolean phase; the distance loop runs in gjk_dist_pass
      o.point_valid = false;
      o.iterations = 0;
      o.p0 = o.p1 = mk3(0, 0, 0);
      const int k = gjk_boolean(sup, -plain, prm.gjk_tol, prm.gjk_max_iter, s, o);
      if (k == kBoolSeparated) {
        if (g.lane == 0) push_dist(dl, pid, s, 0, o.iterations, kStagePlain);
        continue;
      }
      if (k == kBoolUndetermined) o.point_valid = extract_try_sub(s, o.p0, o.p1);
    } else if (MODE == kPassSplitWarm) {
      // the boolean phases of FULL's runs below: the learned direction (a
      // separation certificate within warm_probe supports), else the plain one
      o.point_valid = false;
      o.iterations = 0;
      o.p0 = o.p1 = mk3(0, 0, 0);
      const f3 guess = mk3(__ldg(b.guess + 3 * (size_t)pid), __ldg(b.guess + 3 * (size_t)pid + 1),
                           __ldg(b.guess + 3 * (size_t)pid + 2));
      int k = gjk_boolean(sup, -guess, prm.gjk_tol, prm.gjk_max_iter, s, o, prm.warm_probe);
      int stage = kStageLearned, before = 0;
      if (k != kBoolSeparated && !(o.status == kGjkIntersect && !prm.want_epa)) {
        before = o.iterations;
        o.iterations = 0;
        k = gjk_boolean(sup, -plain, prm.gjk_tol, prm.gjk_max_iter, s, o);
        stage = kStagePlainCertified;
      }
      if (k == kBoolSeparated) {
        if (g.lane == 0) push_dist(dl, pid, s, before, o.iterations, stage);
        continue;
      }
      if (k == kBoolUndetermined) o.point_valid = extract_try_sub(s, o.p0, o.p1);
      o.iterations += before;
    } else if (MODE == kPassFull && b.guess) {
      // Learned direction first, for a separation certificate within
      // warm_probe supports and a distance certified to warm_gap.  A pair it
      // does not settle (overlapping: its EPA must start from the plain
      // simplex; probe exhausted; no certified distance) is rerun from the
      // plain direction with the same certified stop, and a pair that even
      // then gets no certified distance is rerun once more under the
      // reference's own stop.  Every run counts as iterations.
      const f3 guess = mk3(__ldg(b.guess + 3 * (size_t)pid), __ldg(b.guess + 3 * (size_t)pid + 1),
                           __ldg(b.guess + 3 * (size_t)pid + 2));
      o = gjk_evaluate(sup, -guess, prm.gjk_tol, prm.gjk_max_iter, prm.want_distance != 0, s, prm.warm_probe,
                       prm.warm_gap);
      if (!warm_keep(o, prm)) {
        int done_iters = o.iterations;
        o = gjk_evaluate(sup, -plain, prm.gjk_tol, prm.gjk_max_iter, prm.want_distance != 0, s, 0, prm.warm_gap);
        if (uncertified(o, prm)) {
          done_iters += o.iterations;
          o = gjk_evaluate(sup, -plain, prm.gjk_tol, prm.gjk_max_iter, prm.want_distance != 0, s);
        }
        o.iterations += done_iters;
      }
    } else {
      o = gjk_evaluate(sup, -plain, prm.gjk_tol, prm.gjk_max_iter, prm.want_distance != 0, s);
    }
    if (g.lane != 0) continue;
    finish_pair(b, prm, q, pid, o, s);
  }
}


// The distance loop of the separated pairs a SPLIT or SPLIT_WARM gjk_pass
// handed over (gjk_distance.hpp:10-105 from the separating vertex), as a
// persistent grid whose warps take 32 / LANES records at a time from dl.next.
// The stop per record stage, as FULL's runs: the reference's (plain run); the
// certified one (learned start: an uncertified pair goes to the redo list);
// the certified one, then the reference's from the same vertex (plain run of
// a learned-start query).
template <int LANES>
__global__ void __launch_bounds__(128, FCLG_GJK_MINB) gjk_dist_pass(BatchArgs b, QueryParams prm, EpaQueue q,
                                                        DistList dl) {
  const Group<LANES> g = Group<LANES>::make();
  constexpr uint32_t kPer = 32 / LANES;
  const uint32_t slot = (threadIdx.x & 31u) / LANES;
  const uint32_t n = *dl.count;
  auto take = [&]() -> uint32_t {
    uint32_t k = 0;
    if ((threadIdx.x & 31u) == 0) k = atomicAdd(dl.next, kPer);
    return __shfl_sync(0xFFFFFFFFu, k, 0);
  };
  for (uint32_t round = take(); round < n; round = take()) {
    const uint32_t item = round + slot;
    if (item >= n) continue;
    const float4 r0 = dl.rec[3 * (size_t)item], r1 = dl.rec[3 * (size_t)item + 1], r2 = dl.rec[3 * (size_t)item + 2];
    const uint32_t pid = __float_as_uint(r0.x);
    const int stage = __float_as_int(r0.w);
    const PairDev pr = load_pair(b.pairs, pid);
    MinkowskiSupport<LANES> sup;
    sup.A = load_shape(b.shapes, LANES == 1 ? b.walk : nullptr, pr.a);
    sup.B = load_shape(b.shapes, LANES == 1 ? b.walk : nullptr, pr.b);
    sup.pose = pr.pose;
    sup.verts = b.verts;
    sup.hull = b.hull;
    sup.g = g;
    Simplex s;
    GjkOut o;
    o.status = kGjkSeparated;
    o.p0 = o.p1 = mk3(0, 0, 0);
    int before = __float_as_int(r0.y);
    float cert = stage == kStagePlain ? 0.f : prm.warm_gap;
    for (int attempt = 0;; ++attempt) {
      s.set(0, mk3(r1.x, r1.y, r1.z), mk3(r1.w, r2.x, r2.y));
      s.rank = 1;
      o.iterations = __float_as_int(r0.z);
      o.point_valid = min_distance(sup, s, prm.gjk_tol, prm.gjk_max_iter, o.p0, o.p1, o.iterations, cert);
      if (o.point_valid || stage != kStagePlainCertified || attempt > 0) break;
      // not certified: the same run under the reference's stop
      before += o.iterations;
      cert = 0.f;
    }
    if (stage == kStageLearned && !o.point_valid) {
      if (g.lane == 0) {
        const uint32_t r = aggregated_slot(dl.redo_count);
        dl.redo[r] = make_uint2(pid, (uint32_t)o.iterations);
      }
      continue;
    }
    o.iterations += before;
    if (g.lane != 0) continue;
    finish_pair(b, prm, q, pid, o, s);
  }
}

// Learned-start pairs whose distance the learned start did not certify: the
// plain run with the certified stop, then (not certified) with the
// reference's, as FULL runs them; iterations count every run.
template <int LANES>
__global__ void __launch_bounds__(128, FCLG_GJK_MINB) gjk_redo_pass(BatchArgs b, QueryParams prm, EpaQueue q,
                                                        DistList dl) {
  const Group<LANES> g = Group<LANES>::make();
  constexpr uint32_t kPer = 32 / LANES;
  const uint32_t slot = (threadIdx.x & 31u) / LANES;
  const uint32_t n = *dl.redo_count;
  auto take = [&]() -> uint32_t {
    uint32_t k = 0;
    if ((threadIdx.x & 31u) == 0) k = atomicAdd(dl.redo_next, kPer);
    return __shfl_sync(0xFFFFFFFFu, k, 0);
  };
  const f3 plain = mk3(1.f, 0.f, 0.f);
  for (uint32_t round = take(); round < n; round = take()) {
    const uint32_t item = round + slot;
    if (item >= n) continue;
    const uint2 rr = dl.redo[item];
    const uint32_t pid = rr.x;
    const PairDev pr = load_pair(b.pairs, pid);
    MinkowskiSupport<LANES> sup;
    sup.A = load_shape(b.shapes, LANES == 1 ? b.walk : nullptr, pr.a);
    sup.B = load_shape(b.shapes, LANES == 1 ? b.walk : nullptr, pr.b);
    sup.pose = pr.pose;
    sup.verts = b.verts;
    sup.hull = b.hull;
    sup.g = g;
    Simplex s;
    GjkOut o;
    int done_iters = (int)rr.y;
    for (int attempt = 0;; ++attempt) {
      o = gjk_evaluate(sup, -plain, prm.gjk_tol, prm.gjk_max_iter, prm.want_distance != 0, s, 0,
                       attempt == 0 ? prm.warm_gap : 0.f);
      if (attempt > 0 || !uncertified(o, prm)) break;
      done_iters += o.iterations;
    }
    o.iterations += done_iters;
    if (g.lane != 0) continue;
    finish_pair(b, prm, q, pid, o, s);
  }
}

// Launches gjk_pass<LANES, ...> (defined in the translation unit that instantiates LANES): the
// PLAIN variant when the query has no closed-form pairs, MPR or learned start.
template <int LANES>
cudaError_t launch_gjk_lanes(const BatchArgs& b, const QueryParams& prm, const EpaQueue& q, const uint32_t* order,
                             const uint32_t* range, int blocks, cudaStream_t st, uint32_t* next);

#define FCLG_GJK_INSTANTIATE(L)                                                                              \
  template <>                                                                                                \
  cudaError_t launch_gjk_lanes<L>(const BatchArgs& b, const QueryParams& prm, const EpaQueue& q,             \
                                  const uint32_t* order, const uint32_t* range, int blocks, cudaStream_t st, \
                                  uint32_t* next) {                                                          \
    if (FCLG_GJK_PLAIN_VARIANT && !prm.analytic && !prm.use_mpr && !b.guess)                                 \
      gjk_pass<L, kPassPlain><<<blocks, 128, 0, st>>>(b, prm, q, order, range, next, DistList{});            \
    else                                                                                                     \
      gjk_pass<L, kPassFull><<<blocks, 128, 0, st>>>(b, prm, q, order, range, next, DistList{});             \
    return cudaGetLastError();                                                                               \
  }

}  // namespace fclg
