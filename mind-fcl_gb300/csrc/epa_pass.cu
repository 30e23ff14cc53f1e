// EPA pass of a convex query batch: persistent grid, one warp per overlapping
// pair listed by the GJK pass (gjk_pass.cu), polytope in shared memory.
#include "epa.cuh"
#include "kernels.h"

namespace fclg {

// Small layout: 128 faces / 72 vertices (~8.4 KB of shared memory per warp,
// two 13-warp CTAs per SM: 26 warps, the most the SM's shared memory holds,
// at 72 registers -- an SM sub-partition then holds seven warps; measured
// against six 4-warp and five 5-warp CTAs: 9.26 / 9.03 / 8.97 ms on 10^6
// mixed pairs; a polytope of 128 faces has about 66 vertices);
// large layout: the reference's 256 faces (~18 KB per warp, three 4-warp CTAs
// per SM).
#ifndef FCLG_EPA_SMALL_V
#define FCLG_EPA_SMALL_V 72
#endif
#ifndef FCLG_EPA_SMALL_MINB
#define FCLG_EPA_SMALL_MINB 2
#endif
#ifndef FCLG_EPA_SMALL_WARPS
#define FCLG_EPA_SMALL_WARPS 13
#endif
constexpr int kSmallF = 128, kSmallV = FCLG_EPA_SMALL_V, kSmallWarps = FCLG_EPA_SMALL_WARPS,
              kSmallMinB = FCLG_EPA_SMALL_MINB;
#ifndef FCLG_EPA_LARGE_MINB
#define FCLG_EPA_LARGE_MINB 3
#endif
constexpr int kLargeF = 256, kLargeV = 192, kLargeWarps = 4, kLargeMinB = FCLG_EPA_LARGE_MINB;
static_assert(EpaResume<kSmallF, kSmallV>::kBytes <= kEpaResumeBytes, "resume record size");

// EPA over the work list.  The small layout runs every listed pair and hands
// the pairs whose polytope outgrows it to `ovf` (indices into the work list),
// the first ovf.resume_cap of them with their polytope state; the large
// layout continues those from their state and reruns the rest.
template <int FMAX, int VMAX, int WARPS, int MINB>
__global__ void __launch_bounds__(WARPS * 32, MINB) epa_pass(BatchArgs b, QueryParams prm, EpaQueue q,
                                                            EpaQueue ovf, int large) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  EpaSmem<FMAX, VMAX>& P = reinterpret_cast<EpaSmem<FMAX, VMAX>*>(smem_raw)[threadIdx.x >> 5];
  const unsigned lane = threadIdx.x & 31u;
  const uint32_t n = large ? *ovf.count : *q.count;
  const uint32_t gw = blockIdx.x * WARPS + (threadIdx.x >> 5);
  const uint32_t nw = gridDim.x * WARPS;
  // The final layout enforces the requested face limit itself; the small
  // layout runs under the request's limit and overflows at its own capacity.
  const bool final_layout = large || prm.epa_max_faces <= FMAX;
  const int max_faces = (final_layout && prm.epa_max_faces > FMAX) ? FMAX : prm.epa_max_faces;
  // Pairs differ in EPA iterations by an order of magnitude, so each warp
  // takes its next entry from a shared counter as it finishes one, and the
  // warps end together (results do not depend on which warp runs a pair).
  uint32_t* next = large ? ovf.next : q.next;
  auto take = [&](uint32_t done) -> uint32_t {
    if (!next) return done + nw;
    uint32_t k = 0;
    if (lane == 0) k = atomicAdd(next, 1u);
    return __shfl_sync(0xFFFFFFFFu, k, 0);
  };
  for (uint32_t k = next ? take(0) : gw; k < n; k = take(k)) {
    const uint32_t item = large ? ovf.list[k] : k;
    const uint32_t pid = q.list[item];
    const float4* r = q.rec + 7 * (size_t)item;
    float f[28];
#pragma unroll
    for (int j = 0; j < 7; ++j) {
      const float4 v = r[j];
      f[4 * j] = v.x;
      f[4 * j + 1] = v.y;
      f[4 * j + 2] = v.z;
      f[4 * j + 3] = v.w;
    }
    const int rank = __float_as_int(f[0]);
    const int gjk_iters = __float_as_int(f[25]);
    f3 spa[4], spb[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      spa[i] = mk3(f[1 + 6 * i], f[2 + 6 * i], f[3 + 6 * i]);
      spb[i] = mk3(f[4 + 6 * i], f[5 + 6 * i], f[6 + 6 * i]);
    }
    const PairDev pr = load_pair(b.pairs, pid);
    if (lane == 0) {
      P.pair.A = load_shape(b.shapes, pr.a);
      P.pair.B = load_shape(b.shapes, pr.b);
      P.pair.pose = pr.pose;
      P.pair.verts = b.verts;
    }
    __syncwarp();
    const SharedSupport32 sup{&P.pair};
    EpaWarp<FMAX, VMAX, SharedSupport32> E{P, sup, prm.epa_tol, lane, 0, 0, 0, 0, 0u};
    EpaResult er;
    if (large && k < ovf.resume_cap && FMAX >= kSmallF && VMAX >= kSmallV) {
      er = E.template resume<kSmallF, kSmallV>(reinterpret_cast<const unsigned char*>(ovf.rec) +
                                                   (size_t)k * kEpaResumeBytes,
                                               prm.epa_max_iter, max_faces, final_layout);
    } else {
      er = E.run(rank < 1 ? 1 : (rank > 4 ? 4 : rank), spa, spb, prm.epa_max_iter, max_faces, final_layout);
    }
    if (er.status == kEpaOverflow) {
      uint32_t slot = 0;
      if (lane == 0) {
        slot = atomicAdd(ovf.count, 1u);
        ovf.list[slot] = item;
      }
      slot = __shfl_sync(0xFFFFFFFFu, slot, 0);
      if constexpr (FMAX == kSmallF && VMAX == kSmallV) {
        if (slot < ovf.resume_cap)
          E.template save<kSmallF, kSmallV>(reinterpret_cast<unsigned char*>(ovf.rec) + (size_t)slot * kEpaResumeBytes,
                                            er);
      }
    } else if (lane == 0) {
      {
        const int32_t status = kGjkIntersect | ((er.status + 1) << 8);
        const uint32_t iters = (uint32_t)(gjk_iters + er.iterations);
        if (er.status != kEpaFailed) {
          f3 nv = er.p0 - er.p1;
          nv = (sqn(nv) > 0.f) ? normalized(nv) : mk3(0, 0, 1);
          store_result(b.results, pid, -er.depth, nv, er.p0, er.p1, status, iters, true, true);
        } else {
          store_result(b.results, pid, -1.f, mk3(0, 0, 1), mk3(0, 0, 0), mk3(0, 0, 0), status, iters, true, false);
        }
      }
    }
    __syncwarp();
  }
}

size_t epa_smem_bytes() { return (size_t)kSmallWarps * sizeof(EpaSmem<kSmallF, kSmallV>); }
size_t epa_smem_bytes_large() { return (size_t)kLargeWarps * sizeof(EpaSmem<kLargeF, kLargeV>); }

cudaError_t prepare_epa() {
  cudaError_t e = cudaFuncSetAttribute(epa_pass<kSmallF, kSmallV, kSmallWarps, kSmallMinB>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)epa_smem_bytes());
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(epa_pass<kLargeF, kLargeV, kLargeWarps, kLargeMinB>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)epa_smem_bytes_large());
}

cudaError_t launch_epa(const BatchArgs& b, const QueryParams& prm, const EpaQueue& q, const EpaQueue& ovf,
                       int num_sms, int ctas_per_sm, cudaStream_t st) {
  if (b.n_pairs == 0) return cudaSuccess;
  const int small_blocks = num_sms * (ctas_per_sm > 0 ? ctas_per_sm : kSmallMinB);
  epa_pass<kSmallF, kSmallV, kSmallWarps, kSmallMinB>
      <<<small_blocks, kSmallWarps * 32, epa_smem_bytes(), st>>>(b, prm, q, ovf, 0);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || prm.epa_max_faces <= kSmallF) return e;
  epa_pass<kLargeF, kLargeV, kLargeWarps, kLargeMinB>
      <<<num_sms * kLargeMinB, kLargeWarps * 32, epa_smem_bytes_large(), st>>>(b, prm, q, ovf, 1);
  return cudaGetLastError();
}

int epa_max_faces_supported() { return kLargeF; }

int epa_default_ctas_per_sm() { return kSmallMinB; }

}  // namespace fclg
