// Translational continuous collision of shape pairs (fcl::translational_ccd,
// narrowphase/continuous_collision-inl.h:20-37 through
// ShapePairTranslationalCollisionSolver::RunShapePair,
// narrowphase/detail/ccd/shape_pair_ccd-inl.h:57-160), one thread per pair:
// shape a moves along a unit axis of its own frame by a distance; shape b
// stays at the pair's pose.
//
//   * Swept-volume MPR (TranslationalCollisionGJK, ccd/gjk_ccd-inl.h:7-187)
//     in FP32: shape a's support gains the displacement when the direction
//     points along it, its interior point half of it; the boolean is MPR's
//     Intersect, the one-sample time of collision the origin's barycentric
//     weights in the final portal.  Pairs run in shape-class order (the
//     bucketing of the distance query) so that a warp runs one support pair.
//   * Box intervals (BoxPairTranslationalCCD::IsDisjoint, ccd/box_pair_ccd-
//     inl.h:112-393) in FP64 with explicitly rounded operations (no fused
//     multiply-add), so that the decision and the interval equal the FP64
//     restatement's bit for bit: box-box pairs take this test alone
//     (shape_pair_ccd-inl.h:113-133), the approximate request uses it on the
//     shapes' local boxes as a pre-check before MPR (:93-110).
#include "ccd.h"
#include "mpr.cuh"

namespace fclg {
namespace {

// Shape a swept along `sweep` (computeSupport's ShapeSweptVolume case,
// narrowphase/detail/gjk_solver_cvx-inl.h:93-101).
template <class Base>
struct SweptSupport {
  Base base;
  f3 sweep;
  __device__ __forceinline__ void operator()(f3 d, f3& pa, f3& pb) const {
    base(d, pa, pb);
    if (dot(d, sweep) > 0.f) pa = pa + sweep;
  }
};

// FP64 with each operation rounded on its own (the restatement is compiled
// without contraction).
__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmax(double a, double b) { return (a < b) ? b : a; }  // std::max
__device__ __forceinline__ double dmin(double a, double b) { return (b < a) ? b : a; }  // std::min
__device__ __forceinline__ double dot3(double a0, double a1, double a2, double b0, double b1, double b2) {
  return da(da(dm(a0, b0), dm(a1, b1)), dm(a2, b2));
}

struct Iv {
  double lo, hi;
  __device__ void meet(double l, double h) {
    lo = dmax(lo, l);
    hi = dmin(hi, h);
  }
  __device__ bool empty() const { return lo > hi + 0.0; }
};

// CheckEmptyTocIntervalOnAxis, scalar form (box_pair_ccd-inl.h:10-42), unscaled.
__device__ bool axis_empty(double h1, double abs_d, bool pos, double h2, double off, double& lo, double& hi) {
  const double b1_lb = pos ? -h1 : ds(-h1, abs_d);
  const double b1_ub = pos ? da(h1, abs_d) : h1;
  const double b2_lb = ds(off, h2);
  const double b2_ub = da(off, h2);
  if (b1_lb > b2_ub || b2_lb > b1_ub) return true;
  if (pos) {
    lo = dmax(0.0, da(-h1, b2_lb));
    hi = dmin(abs_d, da(h1, b2_ub));
  } else {
    lo = dmax(0.0, ds(-h1, b2_ub));
    hi = dmin(abs_d, ds(h1, b2_lb));
  }
  return false;
}

// Three axes at once, scaled to [0, 1] (box_pair_ccd-inl.h:44-85).
__device__ bool axes3_empty(const double h1[3], const double d[3], const double h2[3], const double off[3],
                            double zero_tol, Iv& out) {
  double b1_lb[3], b1_ub[3], b2_lb[3], b2_ub[3];
  bool pos[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    pos[k] = d[k] > 0.0;
    b1_lb[k] = pos[k] ? -h1[k] : da(-h1[k], d[k]);
    b1_ub[k] = pos[k] ? da(h1[k], d[k]) : h1[k];
    b2_lb[k] = ds(off[k], h2[k]);
    b2_ub[k] = da(off[k], h2[k]);
  }
#pragma unroll
  for (int k = 0; k < 3; ++k)
    if (b1_lb[k] > b2_ub[k] || b2_lb[k] > b1_ub[k]) return true;
  double lo = -INFINITY, hi = INFINITY;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double raw_lo = pos[k] ? da(-h1[k], b2_lb[k]) : ds(-h1[k], b2_ub[k]);
    const double raw_hi = pos[k] ? da(h1[k], b2_ub[k]) : ds(h1[k], b2_lb[k]);
    const double inv = __ddiv_rn(1.0, dmax(fabs(d[k]), zero_tol));
    lo = dmax(lo, dmax(dm(raw_lo, inv), 0.0));
    hi = dmin(hi, dmin(dm(raw_hi, inv), 1.0));
  }
  out.lo = lo;
  out.hi = hi;
  return out.empty();
}

// isDisjointArray (box_pair_ccd-inl.h:112-214): box 1 (half sizes h1) moving
// by u * dist, box 2 (half sizes h2) with rotation R (row-major, box 2 in
// box 1) and centre t in box 1's frame.
__device__ bool box_pair_disjoint(const double h1[3], const double u[3], double dist, const double R[9],
                                  const double t[3], const double h2[3], double zero_tol, Iv& iv) {
  double Ra[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) Ra[k] = fabs(R[k]);
  iv.lo = 0.0;
  iv.hi = 1.0;
  {  // box 1's axes
    double d[3], h2p[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      d[k] = dm(u[k], dist);
      h2p[k] = dot3(Ra[3 * k], Ra[3 * k + 1], Ra[3 * k + 2], h2[0], h2[1], h2[2]);
    }
    Iv a;
    if (axes3_empty(h1, d, h2p, t, zero_tol, a)) return true;
    iv.meet(a.lo, a.hi);
    if (iv.empty()) return true;
  }
  {  // box 2's axes
    double h1p[3], d[3], off[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      h1p[k] = dot3(Ra[k], Ra[3 + k], Ra[6 + k], h1[0], h1[1], h1[2]);
      d[k] = dm(dot3(R[k], R[3 + k], R[6 + k], u[0], u[1], u[2]), dist);
      off[k] = dot3(R[k], R[3 + k], R[6 + k], t[0], t[1], t[2]);
    }
    Iv a;
    if (axes3_empty(h1p, d, h2, off, zero_tol, a)) return true;
    iv.meet(a.lo, a.hi);
    if (iv.empty()) return true;
  }
  for (int k = 0; k < 3; ++k) {
    for (int i = 0; i < 3; ++i) {
      // a = e_k x (column i of R): not unit, possibly zero
      const double c0 = R[i], c1 = R[3 + i], c2 = R[6 + i];
      const double e0 = k == 0 ? 1.0 : 0.0, e1 = k == 1 ? 1.0 : 0.0, e2 = k == 2 ? 1.0 : 0.0;
      const double a0 = ds(dm(e1, c2), dm(e2, c1));
      const double a1 = ds(dm(e2, c0), dm(e0, c2));
      const double a2 = ds(dm(e0, c1), dm(e1, c0));
      const double h1a = dot3(fabs(a0), fabs(a1), fabs(a2), h1[0], h1[1], h1[2]);
      const double off = dot3(a0, a1, a2, t[0], t[1], t[2]);
      const double b0 = dot3(R[0], R[3], R[6], a0, a1, a2);
      const double b1 = dot3(R[1], R[4], R[7], a0, a1, a2);
      const double b2 = dot3(R[2], R[5], R[8], a0, a1, a2);
      const double h2a = dot3(fabs(b0), fabs(b1), fabs(b2), h2[0], h2[1], h2[2]);
      const double proj = dot3(a0, a1, a2, u[0], u[1], u[2]);
      const bool pos = proj > 0.0;
      const double abs_d = pos ? dm(proj, dist) : dm(-proj, dist);
      double lo, hi;
      if (axis_empty(h1a, abs_d, pos, h2a, off, lo, hi)) return true;
      // ScaleIntervalBoxDisjoint (box_pair_ccd-inl.h:99-110)
      if (abs_d < zero_tol) {
        lo = 0.0;
        hi = 1.0;
      } else {
        lo = __ddiv_rn(lo, abs_d);
        hi = __ddiv_rn(hi, abs_d);
      }
      iv.meet(lo, hi);
      if (iv.empty()) return true;
    }
  }
  return false;
}

// A shape's local box: half sizes and centre (computeLocalAABB; a hull's from
// the precomputed vertex extent).
__device__ void local_box(const ShapeDev& s, uint32_t id, const float4* __restrict__ aabb, double h[3],
                          double c[3]) {
  c[0] = c[1] = c[2] = 0.0;
  switch (s.type) {
    case kBox: h[0] = s.p0; h[1] = s.p1; h[2] = s.p2; return;
    case kSphere: h[0] = h[1] = h[2] = s.p0; return;
    case kCapsule: h[0] = h[1] = s.p0; h[2] = da((double)s.p1, (double)s.p0); return;
    case kCylinder: h[0] = h[1] = s.p0; h[2] = s.p1; return;
    default: {
      const float4 lo = __ldg(aabb + 2 * (size_t)id), hi = __ldg(aabb + 2 * (size_t)id + 1);
      const double l[3] = {lo.x, lo.y, lo.z}, u[3] = {hi.x, hi.y, hi.z};
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        h[k] = dm(ds(u[k], l[k]), 0.5);
        c[k] = dm(da(l[k], u[k]), 0.5);
      }
    }
  }
}

// convertBV(local AABB, pose) of both shapes, then IsDisjoint
// (box_pair_ccd-inl.h:365-393) with box 1 at its frame's axes.
__device__ bool obb_pair_disjoint(const ShapeDev& A, uint32_t ia, const ShapeDev& B, uint32_t ib, const Pose& pose,
                                  const double u[3], double dist, const float4* __restrict__ aabb, double zero_tol,
                                  Iv& iv) {
  double h1[3], c1[3], h2[3], c2[3];
  local_box(A, ia, aabb, h1, c1);
  local_box(B, ib, aabb, h2, c2);
  double R[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) R[k] = pose.r[k];
  const double pt[3] = {pose.t.x, pose.t.y, pose.t.z};
  double t[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) t[k] = ds(da(dot3(R[3 * k], R[3 * k + 1], R[3 * k + 2], c2[0], c2[1], c2[2]), pt[k]), c1[k]);
  return box_pair_disjoint(h1, u, dist, R, t, h2, zero_tol, iv);
}

// computeOneTocSampleForIntersection (gjk_ccd-inl.h:106-187), in FP32 like
// the portal it reads.
__device__ float toc_sample(const MprPortal& P, f3 sweep) {
  constexpr float kV0Phase = 0.5f;
  if (P.count < 1) return kV0Phase;
  auto phase = [&](f3 d) { return dot(d, sweep) > 0.f ? 1.f : 0.f; };
  if (P.count < 3) {
    const float n0 = sqrtf(sqn(P.v0)), n1 = sqrtf(sqn(P.v1));
    const float n01 = n0 + n1;
    if (n01 <= 0.f) return kV0Phase;
    return (n1 * kV0Phase + n0 * phase(P.d1)) / n01;
  }
  const f3 a1 = P.v1 - P.v0, a2 = P.v2 - P.v0, a3 = P.v3 - P.v0;
  const float o012 = fabsf(dot(cross(a1, a2), P.v0));
  const float o013 = fabsf(dot(cross(a1, a3), P.v0));
  const float o023 = fabsf(dot(cross(a2, a3), P.v0));
  const float o123 = fabsf(dot(cross(P.v2 - P.v1, P.v3 - P.v1), P.v1));
  const float total = ((o012 + o013) + o023) + o123;
  if (total <= 0.f) return 0.f;
  return (((o123 * kV0Phase + o023 * phase(P.d1)) + o013 * phase(P.d2)) + o012 * phase(P.d3)) / total;
}

#ifndef FCLG_CCD_MINB
#define FCLG_CCD_MINB 5
#endif

__global__ void __launch_bounds__(128, FCLG_CCD_MINB) ccd_pass(BatchArgs b, const float4* __restrict__ disp,
                                                   const float4* __restrict__ aabb, CcdParams prm,
                                                   const uint32_t* __restrict__ order, float4* __restrict__ out,
                                                   uint32_t* next) {
  // a warp runs 32 pairs at a time; with a counter (next, zero before the
  // launch) it takes its next 32 there as it finishes, so the persistent
  // grid's warps end together
  const unsigned lane = threadIdx.x & 31u;
  const uint32_t n_warps = (gridDim.x * blockDim.x) >> 5;
  auto take = [&](uint32_t done) -> uint32_t {
    if (!next) return done + n_warps * 32u;
    uint32_t r = 0;
    if (lane == 0) r = atomicAdd(next, 32u);
    return __shfl_sync(0xFFFFFFFFu, r, 0);
  };
  const uint32_t first = next ? take(0) : ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32u;
  for (uint32_t round = first; round < b.n_pairs; round = take(round)) {
    const uint32_t k = round + lane;
    if (k >= b.n_pairs) continue;
    const uint32_t pid = order ? __ldg(order + k) : k;
    const PairDev pr = load_pair(b.pairs, pid);
    uint32_t st = kCcdNoMpr;
    bool hit = false;
    float lo = -1.f, hi = -1.f;
    if (pr.a >= b.n_shapes || pr.b >= b.n_shapes) {
      out[pid] = make_float4(__uint_as_float(0u), __uint_as_float(st | kCcdBadShape), lo, hi);
      continue;
    }
    const float4 dq = __ldg(disp + pid);
    const double u[3] = {dq.x, dq.y, dq.z};
    const double dist = dq.w;
    MinkowskiSupport<1> ms;
    ms.A = load_shape(b.shapes, b.walk, pr.a);
    ms.B = load_shape(b.shapes, b.walk, pr.b);
    ms.pose = pr.pose;
    ms.verts = b.verts;
    ms.hull = b.hull;
    ms.g = Group<1>::make();
    const bool boxes = ms.A.type == kBox && ms.B.type == kBox;
    bool run_mpr = !boxes;
    if (boxes || prm.toc_type == kTocBox) {
      Iv iv;
      st |= kCcdBoxTested;
      const bool disjoint = obb_pair_disjoint(ms.A, pr.a, ms.B, pr.b, pr.pose, u, dist, aabb, prm.zero_tol, iv);
      if (disjoint) {
        st |= kCcdBoxDisjoint;
        run_mpr = false;
      } else {
        lo = (float)iv.lo;
        hi = (float)iv.hi;
        hit = boxes;
      }
    }
    if (run_mpr) {
      SweptSupport<MinkowskiSupport<1>> sup{ms, mk3(dq.x * dq.w, dq.y * dq.w, dq.z * dq.w)};
      Mpr<SweptSupport<MinkowskiSupport<1>>> mpr{sup, prm.max_iter, prm.tol};
      const f3 v0 = (load_interior(b.shapes, pr.a, ms.A.type) + sup.sweep * 0.5f) -
                    pr.pose.apply(load_interior(b.shapes, pr.b, ms.B.type));
      MprPortal P;
      const MprStatus r = mpr.intersect<true>(v0, &P);
      st = (st & ~kCcdNoMpr) | (uint32_t)r;
      hit = r == MprStatus::Intersect;
      if (!hit) {
        lo = hi = -1.f;
      } else if (prm.toc_type == kTocSample) {
        lo = hi = toc_sample(P, sup.sweep);
      }
    }
    out[pid] = make_float4(__uint_as_float(hit ? 1u : 0u), __uint_as_float(st), lo, hi);
  }
}

// Local AABB of every hull (its vertex extent), 2 float4 per shape; other
// shapes' boxes come from their parameters in the pass.
__global__ void hull_aabb_kernel(const int4* __restrict__ shapes, const float4* __restrict__ verts, uint32_t n,
                                 float4* __restrict__ aabb) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const ShapeDev s = load_shape(shapes, i);
    float4 lo = make_float4(0.f, 0.f, 0.f, 0.f), hi = lo;
    if (s.type == kConvex && s.nv > 0) {
      lo = make_float4(INFINITY, INFINITY, INFINITY, 0.f);
      hi = make_float4(-INFINITY, -INFINITY, -INFINITY, 0.f);
      for (uint32_t k = 0; k < s.nv; ++k) {
        const float4 q = __ldg(verts + s.vofs + k);
        lo = make_float4(fminf(lo.x, q.x), fminf(lo.y, q.y), fminf(lo.z, q.z), 0.f);
        hi = make_float4(fmaxf(hi.x, q.x), fmaxf(hi.y, q.y), fmaxf(hi.z, q.z), 0.f);
      }
    }
    aabb[2 * (size_t)i] = lo;
    aabb[2 * (size_t)i + 1] = hi;
  }
}

}  // namespace

cudaError_t launch_hull_aabbs(const int4* shapes, const float4* verts, uint32_t n_shapes, float4* aabb,
                              cudaStream_t st) {
  if (n_shapes == 0) return cudaSuccess;
  const int tb = 256;
  hull_aabb_kernel<<<(int)((n_shapes + tb - 1) / tb), tb, 0, st>>>(shapes, verts, n_shapes, aabb);
  return cudaGetLastError();
}

cudaError_t launch_ccd(const BatchArgs& b, const float4* disp, const float4* aabb, const CcdParams& prm,
                       const uint32_t* order, float4* out, int num_sms, cudaStream_t st, uint32_t* next) {
  if (b.n_pairs == 0) return cudaSuccess;
  // persistent: FCLG_CCD_MINB CTAs on every SM
  ccd_pass<<<num_sms * FCLG_CCD_MINB, 128, 0, st>>>(b, disp, aabb, prm, order, out, next);
  return cudaGetLastError();
}

}  // namespace fclg
