// EPA pass of a convex query batch: persistent grid, one warp per overlapping
// pair listed by the GJK pass (gjk_pass.cu), polytope in shared memory.  The
// warps leave the final FP64 closest-face solve of each pair to a third
// launch that runs it a thread per pair (epa_finalize): on one lane of the
// warp it held the warp for hundreds of FP64 instructions, each of which
// occupies the narrow FP64 pipe as long as a full warp's would.
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

// Final-solve record of a work-list entry, written over the entry's GJK
// simplex record (q.rec, 7 float4) once the entry is done:
//   {wa, pid} {wb, status} {wc, iterations} {pa_a, fb.x} {pa_b, fb.y}
//   {pa_c, fb.z} {fa, pending}
// w* the final face's Minkowski vertices, pa_* their support points on shape
// a, (fa, fb) the fallback support pair; pending 1: epa_finalize solves and
// stores the result, 0: the pass stored it.
constexpr int kFinPending = 6;

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
    EpaWarp<FMAX, VMAX, SharedSupport32, true> E{P, sup, prm.epa_tol, lane, 0, 0, 0, 0, 0u};
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
      const int32_t status = kGjkIntersect | ((er.status + 1) << 8);
      const uint32_t iters = (uint32_t)(gjk_iters + er.iterations);
      float4* fin = q.rec + 7 * (size_t)item;
      if (er.status != kEpaFailed && er.fin_fv != kNoSlot) {
        const uint32_t ia = fvert(er.fin_fv, 0), ib = fvert(er.fin_fv, 1), ic = fvert(er.fin_fv, 2);
        const float4 wa = P.vw[ia], wb = P.vw[ib], wc = P.vw[ic];
        const float4 qa = P.vpa[ia], qb = P.vpa[ib], qc = P.vpa[ic];
        fin[0] = make_float4(wa.x, wa.y, wa.z, __uint_as_float(pid));
        fin[1] = make_float4(wb.x, wb.y, wb.z, __int_as_float(status));
        fin[2] = make_float4(wc.x, wc.y, wc.z, __uint_as_float(iters));
        fin[3] = make_float4(qa.x, qa.y, qa.z, er.p1.x);
        fin[4] = make_float4(qb.x, qb.y, qb.z, er.p1.y);
        fin[5] = make_float4(qc.x, qc.y, qc.z, er.p1.z);
        fin[kFinPending] = make_float4(er.p0.x, er.p0.y, er.p0.z, __int_as_float(1));
      } else {
        if (er.status != kEpaFailed) {
          f3 nv = er.p0 - er.p1;
          nv = (sqn(nv) > 0.f) ? normalized(nv) : mk3(0, 0, 1);
          store_result(b.results, pid, -er.depth, nv, er.p0, er.p1, status, iters, true, true);
        } else {
          store_result(b.results, pid, -1.f, mk3(0, 0, 1), mk3(0, 0, 0), mk3(0, 0, 0), status, iters, true, false);
        }
        fin[kFinPending] = make_float4(0.f, 0.f, 0.f, __int_as_float(0));
      }
    }
    __syncwarp();
  }
}

// The final solves the EPA launches left, a thread per work-list entry
// (epa_final_solve, then the result record as the pass writes it).
__global__ void __launch_bounds__(256) epa_finalize(BatchArgs b, EpaQueue q) {
  const uint32_t n = *q.count;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const float4* fin = q.rec + 7 * (size_t)k;
    const float4 f6 = fin[kFinPending];
    if (__float_as_int(f6.w) != 1) continue;
    const float4 f0 = fin[0], f1 = fin[1], f2 = fin[2], f3r = fin[3], f4 = fin[4], f5 = fin[5];
    EpaResult er;
    epa_final_solve(ld3(f0), ld3(f1), ld3(f2), ld3(f3r), ld3(f4), ld3(f5), ld3(f6), mk3(f3r.w, f4.w, f5.w), er.p0,
                    er.p1, er.depth);
    f3 nv = er.p0 - er.p1;
    nv = (sqn(nv) > 0.f) ? normalized(nv) : mk3(0, 0, 1);
    store_result(b.results, __float_as_uint(f0.w), -er.depth, nv, er.p0, er.p1, __float_as_int(f1.w),
                 __float_as_uint(f2.w), true, true);
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
  if (e == cudaSuccess && prm.epa_max_faces > kSmallF) {
    epa_pass<kLargeF, kLargeV, kLargeWarps, kLargeMinB>
        <<<num_sms * kLargeMinB, kLargeWarps * 32, epa_smem_bytes_large(), st>>>(b, prm, q, ovf, 1);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) return e;
  epa_finalize<<<num_sms * 4, 256, 0, st>>>(b, q);
  return cudaGetLastError();
}

int epa_launches(const QueryParams& prm) { return prm.epa_max_faces > kSmallF ? 3 : 2; }

int epa_max_faces_supported() { return kLargeF; }

int epa_default_ctas_per_sm() { return kSmallMinB; }

}  // namespace fclg
