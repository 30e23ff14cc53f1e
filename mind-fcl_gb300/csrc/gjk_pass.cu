// GJK pass launcher: picks the lane count's instantiation (gjk_pass_l*.cu),
// or the refilling one-lane pass defined here.
#include <algorithm>

#include "gjk_pass.cuh"

namespace fclg {

FCLG_GJK_INSTANTIATE(1)
FCLG_GJK_INSTANTIATE(2)

// Free lanes of a warp that trigger a refill of them all.
constexpr int kRefillBatch = 8;
// CTAs per SM the refilling pass is compiled for (its register budget) and launched with.
#ifndef FCLG_REFILL_MINB
#define FCLG_REFILL_MINB 4
#endif

// One lane per pair, pairs refilled per lane: every lane of a warp steps its
// own pair's GJK run one support evaluation at a time (GjkRun), and a lane
// whose pair is done takes the next one from its warp's share of the items
// (warp w takes items 32 (w + k W) .. 32 (w + k W) + 31, k = 0, 1, ...,
// W warps in the grid, in the order its lanes come free).  A warp's lanes so
// stay busy until its share runs out, instead of each round of 32 pairs
// waiting for its slowest pair -- which is also what lets a learned warm
// start's shorter runs shorten the pass.  For queries without MPR or
// closed-form pairs; the results equal gjk_pass<1>'s (the same decisions).
__global__ void __launch_bounds__(128, FCLG_REFILL_MINB) gjk_refill(BatchArgs b, QueryParams prm, EpaQueue q,
                                                               const uint32_t* __restrict__ order,
                                                               const uint32_t* __restrict__ range) {
  uint32_t begin = 0, end = b.n_pairs;
  if (range) {
    begin = range[0];
    end = range[1];
  }
  const unsigned lane = threadIdx.x & 31u;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t n_warps = (gridDim.x * blockDim.x) >> 5;
  const Group<1> g = Group<1>::make();
  // GJKSolver's default guess (1, 0, 0), gjk_solver-inl.h:1129
  const f3 plain = mk3(1.f, 0.f, 0.f);
  MinkowskiSupport<1> sup;
  sup.verts = b.verts;
  sup.hull = b.hull;
  sup.g = g;
  GjkRun run;
  uint32_t pid = 0;
  bool live = false;
  int stage = 0;       // 0 plain run; with a learned start: 1 learned, 2 plain certified, then 0
  int done_iters = 0;  // iterations of the pair's earlier runs
  uint32_t next = 0;  // warp-uniform: next unassigned position in the warp's share
  for (;;) {
    unsigned want = __ballot_sync(0xFFFFFFFFu, !live);
    // refill in batches: the loads of a new pair stall the whole warp, so
    // wait until a quarter of the lanes are free (or none is busy)
    if (__popc(want) < kRefillBatch && want != 0xFFFFFFFFu) want = 0;
    if (want & (1u << lane)) {
      const uint32_t k = next + (uint32_t)__popc(want & ((1u << lane) - 1u));
      const uint64_t item = (uint64_t)begin + ((uint64_t)(k >> 5) * n_warps + warp) * 32u + (k & 31u);
      if (item < end) {
        pid = order ? order[item] : (uint32_t)item;
        const PairDev pr = load_pair(b.pairs, pid);
        if (pr.a >= b.n_shapes || pr.b >= b.n_shapes) {
          store_invalid(b.results, pid);
        } else {
          sup.A = load_shape(b.shapes, b.walk, pr.a);
          sup.B = load_shape(b.shapes, b.walk, pr.b);
          sup.pose = pr.pose;
          stage = b.guess != nullptr ? 1 : 0;
          done_iters = 0;
          if (stage == 1) {
            const f3 guess = mk3(__ldg(b.guess + 3 * (size_t)pid), __ldg(b.guess + 3 * (size_t)pid + 1),
                                 __ldg(b.guess + 3 * (size_t)pid + 2));
            run.begin(-guess, prm.warm_probe, prm.warm_gap);
          } else {
            run.begin(-plain);
          }
          live = true;
        }
      }
    }
    next += (uint32_t)__popc(want);
    if (__all_sync(0xFFFFFFFFu, !live)) {
      // no lane holds a pair: stop once the warp's next position is past the share
      const uint64_t first = (uint64_t)begin + ((uint64_t)(next >> 5) * n_warps + warp) * 32u + (next & 31u);
      if (first >= end) break;
      continue;
    }
    if (live && run.step(sup, prm.gjk_tol, prm.gjk_max_iter, prm.want_distance != 0)) {
      const GjkOut& o = run.o;
      // the same three runs as gjk_pass: learned (kept on warm_keep), plain
      // certified (kept unless uncertified), plain under the reference's stop
      if (stage == 1 && !warm_keep(o, prm)) {
        stage = 2;
        done_iters += o.iterations;
        run.begin(-plain, 0, prm.warm_gap);
      } else if (stage == 2 && uncertified(o, prm)) {
        stage = 0;
        done_iters += o.iterations;
        run.begin(-plain);
      } else {
        GjkOut out = o;
        out.iterations += done_iters;
        finish_pair(b, prm, q, pid, out, run.s);
        live = false;
      }
    }
  }
}


int gjk_default_ctas_per_sm() { return FCLG_GJK_MINB; }

bool gjk_split_applies(const BatchArgs& b, const QueryParams& prm, int lanes, int blocks, bool refill) {
  // the one-lane plain distance pass on a persistent grid (the distance
  // launch sizes itself by a count on the device)
  return FCLG_GJK_PLAIN_VARIANT && lanes == 1 && blocks > 0 && !refill && !prm.analytic && !prm.use_mpr &&
         prm.want_distance;
}

int gjk_split_launches(const BatchArgs& b, const QueryParams& prm, int lanes, int blocks, bool refill) {
  if (!gjk_split_applies(b, prm, lanes, blocks, refill)) return 1;
  return b.guess ? 3 : 2;
}

cudaError_t launch_gjk(const BatchArgs& b, const QueryParams& prm, const EpaQueue& q, int lanes,
                       const uint32_t* order, const uint32_t* range, int blocks, cudaStream_t st, bool refill,
                       uint32_t* next, const DistList* dl) {
  if (b.n_pairs == 0) return cudaSuccess;
  if (dl && gjk_split_applies(b, prm, lanes, blocks, refill)) {
    if (b.guess) gjk_pass<1, kPassSplitWarm><<<blocks, 128, 0, st>>>(b, prm, q, order, range, next, *dl);
    else gjk_pass<1, kPassSplit><<<blocks, 128, 0, st>>>(b, prm, q, order, range, next, *dl);
    gjk_dist_pass<1><<<blocks, 128, 0, st>>>(b, prm, q, *dl);
    if (b.guess) gjk_redo_pass<1><<<blocks, 128, 0, st>>>(b, prm, q, *dl);
    return cudaGetLastError();
  }
  const int threads = 128;
  if (blocks <= 0) {
    const uint64_t total = (uint64_t)b.n_pairs * (uint64_t)lanes;
    blocks = (int)((total + threads - 1) / threads);
    next = nullptr;  // one CTA per 128 lanes of work: the block scheduler balances the grid
  }
  if (refill && lanes == 1 && !prm.use_mpr && !prm.analytic) {
    // a persistent grid: FCLG_REFILL_MINB CTAs on every SM
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess)
      return cudaGetLastError();
    const int grid = std::min<int>(blocks, sms * FCLG_REFILL_MINB);
    gjk_refill<<<grid > 0 ? grid : 1, threads, 0, st>>>(b, prm, q, order, range);
    return cudaGetLastError();
  }
  switch (lanes) {
    case 1: return launch_gjk_lanes<1>(b, prm, q, order, range, blocks, st, next);
    case 2: return launch_gjk_lanes<2>(b, prm, q, order, range, blocks, st, next);
    case 4: return launch_gjk_lanes<4>(b, prm, q, order, range, blocks, st, next);
    case 8: return launch_gjk_lanes<8>(b, prm, q, order, range, blocks, st, next);
    case 16: return launch_gjk_lanes<16>(b, prm, q, order, range, blocks, st, next);
    case 32: return launch_gjk_lanes<32>(b, prm, q, order, range, blocks, st, next);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace fclg
