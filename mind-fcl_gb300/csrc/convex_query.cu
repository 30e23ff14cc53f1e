// The two passes of a convex query batch.
//
//  gjk_pass   one group of LANES lanes per pair: GJK boolean and, for
//             separated pairs, the GJK separation distance; overlapping pairs
//             are appended (warp-aggregated atomics) to a compact work list
//             with their final simplex.
//  epa_pass   persistent grid, one warp per listed pair: EPA from the simplex.
//
// Both passes are stream-ordered and need no host round trip between them:
// the EPA grid reads the list length from device memory, so the pair of
// launches can be captured into a CUDA graph.
#include "epa.cuh"
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

#ifndef FCLG_GJK_MINB
#define FCLG_GJK_MINB 4
#endif
template <int LANES>
__global__ void __launch_bounds__(128, FCLG_GJK_MINB) gjk_pass(BatchArgs b, QueryParams prm, EpaQueue q,
                                                   const uint32_t* __restrict__ order,
                                                   const uint32_t* __restrict__ range) {
  uint32_t begin = 0, end = b.n_pairs;
  if (range) {
    begin = range[0];
    end = range[1];
  }
  const Group<LANES> g = Group<LANES>::make();
  const uint32_t stride = gridDim.x * (blockDim.x / LANES);
  for (uint32_t item = begin + (blockIdx.x * blockDim.x + threadIdx.x) / LANES; item < end; item += stride) {
    const uint32_t pid = order ? order[item] : item;
    const PairDev pr = load_pair(b.pairs, pid);
    if (pr.a >= b.n_shapes || pr.b >= b.n_shapes) {
      if (g.lane == 0) store_invalid(b.results, pid);
      continue;
    }
    MinkowskiSupport<LANES> sup;
    sup.A = load_shape(b.shapes, pr.a);
    sup.B = load_shape(b.shapes, pr.b);
    sup.pose = pr.pose;
    sup.verts = b.verts;
    sup.g = g;
    // GJKSolver's default guess (1, 0, 0), gjk_solver-inl.h:1129
    const f3 plain = mk3(1.f, 0.f, 0.f);
    int mpr_iters = 0;
    if (prm.use_mpr) {
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
    if (b.guess) {
      // Learned direction first.  Overlapping pairs (their EPA must start
      // from the plain simplex) and pairs without a separation certificate
      // are rerun from the plain direction; both runs count as iterations.
      const f3 guess = mk3(__ldg(b.guess + 3 * (size_t)pid), __ldg(b.guess + 3 * (size_t)pid + 1),
                           __ldg(b.guess + 3 * (size_t)pid + 2));
      o = gjk_evaluate(sup, -guess, prm.gjk_tol, prm.gjk_max_iter, prm.want_distance != 0, s);
      const bool keep = (o.status == kGjkSeparated && (o.point_valid || !prm.want_distance)) ||
                        (o.status == kGjkIntersect && !prm.want_epa);
      if (!keep) {
        const int warm_iters = o.iterations;
        o = gjk_evaluate(sup, -plain, prm.gjk_tol, prm.gjk_max_iter, prm.want_distance != 0, s);
        o.iterations += warm_iters;
      }
    } else {
      o = gjk_evaluate(sup, -plain, prm.gjk_tol, prm.gjk_max_iter, prm.want_distance != 0, s);
    }
    if (g.lane != 0) continue;
    if (o.status == kGjkIntersect) {
      if (prm.want_epa) {
        const uint32_t slot = aggregated_slot(q.count);
        q.list[slot] = pid;
        write_simplex(q.rec, slot, s, o.iterations);
        continue;
      }
      store_result(b.results, pid, 0.f, mk3(0, 0, 1), mk3(0, 0, 0), mk3(0, 0, 0), kGjkIntersect,
                   (uint32_t)o.iterations, true, true);
      continue;
    }
    if (!prm.want_distance) {
      store_result(b.results, pid, 0.f, mk3(0, 0, 1), mk3(0, 0, 0), mk3(0, 0, 0), o.status, (uint32_t)o.iterations,
                   false, o.status == kGjkSeparated);
      continue;
    }
    // shapeSignedDistance: valid only for a separation certificate with valid points
    const bool ok = (o.status == kGjkSeparated) && o.point_valid;
    const f3 dv = o.p1 - o.p0;
    const float dist = ok ? nrm(dv) : -1.f;
    f3 nrmv = normalized(dv);
    if (!(sqn(nrmv) > 0.f)) nrmv = mk3(0, 0, 1);
    store_result(b.results, pid, dist, nrmv, o.p0, o.p1, o.status, (uint32_t)o.iterations, false, ok);
  }
}

// EPA over the work list.  The small layout runs every listed pair and hands
// the pairs whose polytope outgrows it to `ovf` (indices into the work list);
// the large layout reruns those.
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
  for (uint32_t k = gw; k < n; k += nw) {
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
    MinkowskiSupport<32> sup;
    sup.A = load_shape(b.shapes, pr.a);
    sup.B = load_shape(b.shapes, pr.b);
    sup.pose = pr.pose;
    sup.verts = b.verts;
    sup.g = Group<32>::make();
    EpaWarp<FMAX, VMAX> E{P, sup, prm.epa_tol, lane, 0, 0, 0, 0, 0u};
    const EpaResult er =
        E.run(rank < 1 ? 1 : (rank > 4 ? 4 : rank), spa, spb, prm.epa_max_iter, max_faces, final_layout);
    if (lane == 0) {
      if (er.status == kEpaOverflow) {
        const uint32_t slot = atomicAdd(ovf.count, 1u);
        ovf.list[slot] = item;
      } else {
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

// Small layout: 128 faces / 128 vertices (~10 KB of shared memory per warp,
// five 4-warp CTAs per SM); large layout: the reference's 256 faces (~18 KB per
// warp, three 4-warp CTAs per SM).
constexpr int kSmallF = 128, kSmallV = 128, kSmallWarps = 4, kSmallMinB = 5;
#ifndef FCLG_EPA_LARGE_MINB
#define FCLG_EPA_LARGE_MINB 3
#endif
constexpr int kLargeF = 256, kLargeV = 192, kLargeWarps = 4, kLargeMinB = FCLG_EPA_LARGE_MINB;

size_t epa_smem_bytes() { return (size_t)kSmallWarps * sizeof(EpaSmem<kSmallF, kSmallV>); }
size_t epa_smem_bytes_large() { return (size_t)kLargeWarps * sizeof(EpaSmem<kLargeF, kLargeV>); }

cudaError_t launch_gjk(const BatchArgs& b, const QueryParams& prm, const EpaQueue& q, int lanes,
                       const uint32_t* order, const uint32_t* range, int blocks, cudaStream_t st) {
  if (b.n_pairs == 0) return cudaSuccess;
  const int threads = 128;
  if (blocks <= 0) {
    const uint64_t total = (uint64_t)b.n_pairs * (uint64_t)lanes;
    blocks = (int)((total + threads - 1) / threads);
  }
  switch (lanes) {
    case 1: gjk_pass<1><<<blocks, threads, 0, st>>>(b, prm, q, order, range); break;
    case 2: gjk_pass<2><<<blocks, threads, 0, st>>>(b, prm, q, order, range); break;
    case 4: gjk_pass<4><<<blocks, threads, 0, st>>>(b, prm, q, order, range); break;
    case 8: gjk_pass<8><<<blocks, threads, 0, st>>>(b, prm, q, order, range); break;
    case 16: gjk_pass<16><<<blocks, threads, 0, st>>>(b, prm, q, order, range); break;
    case 32: gjk_pass<32><<<blocks, threads, 0, st>>>(b, prm, q, order, range); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

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

}  // namespace fclg
