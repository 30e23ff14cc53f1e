// OBB BVH vs OBB BVH boolean collision of two triangle meshes for a batch of
// relative poses: one warp per pose.
//
// Restates OrientedNodeBVHSolver::MeshIntersect
// (narrowphase/detail/traversal/collision/bvh_solver-inl.h:74-164) with the
// penetration request off: node pairs whose boxes overlap (OBB overlap,
// math/bv/OBB-inl.h:305-436) descend into the node with the larger box
// (|extent|^2, OBB-inl.h:153-156), leaf pairs run the 17-axis triangle test
// (intersect-inl.h:723-795, project6 :1082-1102), and a pose stops once it has
// max_contacts contacts (CollisionResult::addContact /
// terminationConditionSatisfied).
//
// GPU layout: the warp keeps its node pairs on a stack in shared memory and
// pops up to 32 per round, one per lane — a depth-first order, 32 wide, that
// keeps the stack short and finds a first contact early.  Children are pushed
// with a warp prefix sum.  Box tests run in FP32 with an added slack that
// covers FP32 rounding, so they never prune a pair the FP64 test keeps.  The
// triangle test runs in FP32 and is re-decided in FP64 whenever an axis sits
// within its rounding bound of the separation threshold, so every
// triangle-pair verdict equals the FP64 one.  A stack that would overflow ends
// the pose with the incomplete bit set in its status.
#include "kernels.h"
#include "mesh_common.cuh"
#include "mesh_kernels.h"

namespace fclg {

namespace {

constexpr int kMeshStack = 1024;
constexpr int kMeshWarps = 4;
constexpr int kMaxRounds = 1 << 22;  // bound against a corrupted tree

struct MeshSmem {
  uint32_t na[kMeshStack];
  uint32_t nb[kMeshStack];
  uint32_t found;
};

// The 17 axes of intersect_Triangle in the order the reference tries them.
template <class V, class Cross>
__device__ __forceinline__ void tri_axes(const V& e1, const V& e2, const V& e3, const V& f1, const V& f2, const V& f3,
                                         V* ax, Cross crs) {
  const V n1 = crs(e1, e2), m1 = crs(f1, f2);
  ax[0] = n1;
  ax[1] = m1;
  ax[2] = crs(e1, f1); ax[3] = crs(e1, f2); ax[4] = crs(e1, f3);
  ax[5] = crs(e2, f1); ax[6] = crs(e2, f2); ax[7] = crs(e2, f3);
  ax[8] = crs(e3, f1); ax[9] = crs(e3, f2); ax[10] = crs(e3, f3);
  ax[11] = crs(e1, n1); ax[12] = crs(e2, n1); ax[13] = crs(e3, n1);
  ax[14] = crs(f1, m1); ax[15] = crs(f2, m1); ax[16] = crs(f3, m1);
}

// FP64 triangle test, the reference's arithmetic (Q posed by the pose).
__device__ bool tri_tri_fp64(const Pose& P, f3 A0, f3 A1, f3 A2, f3 B0, f3 B1, f3 B2) {
  double R[9];
  for (int i = 0; i < 9; ++i) R[i] = P.r[i];
  const d3 T = tod(P.t);
  auto xf = [&](f3 q) {
    return d3{R[0] * q.x + R[1] * q.y + R[2] * q.z + T.x, R[3] * q.x + R[4] * q.y + R[5] * q.z + T.y,
              R[6] * q.x + R[7] * q.y + R[8] * q.z + T.z};
  };
  const d3 P1 = tod(A0);
  const d3 p1{0, 0, 0}, p2 = tod(A1) - P1, p3 = tod(A2) - P1;
  const d3 q1 = xf(B0) - P1, q2 = xf(B1) - P1, q3 = xf(B2) - P1;
  d3 ax[17];
  tri_axes(p2 - p1, p3 - p2, p1 - p3, q2 - q1, q3 - q2, q1 - q3, ax, [](d3 x, d3 y) { return cross(x, y); });
  for (int i = 0; i < 17; ++i) {
    const double P1v = dot(ax[i], p1), P2v = dot(ax[i], p2), P3v = dot(ax[i], p3);
    const double Q1v = dot(ax[i], q1), Q2v = dot(ax[i], q2), Q3v = dot(ax[i], q3);
    const double mn1 = fmin(P1v, fmin(P2v, P3v)), mx1 = fmax(P1v, fmax(P2v, P3v));
    const double mn2 = fmin(Q1v, fmin(Q2v, Q3v)), mx2 = fmax(Q1v, fmax(Q2v, Q3v));
    if (mn1 > mx2 || mn2 > mx1) return false;
  }
  return true;
}

// FP32 triangle test; any axis whose verdict is within the FP32 error bound
// of its threshold sends the pair to the FP64 test.  The bound of axis
// u x v scales with |u| |v| (not |u x v|): for nearly parallel edges the
// computed direction itself carries that error.
__device__ bool tri_tri(const Pose& P, f3 A0, f3 A1, f3 A2, f3 B0, f3 B1, f3 B2) {
  const f3 Q0 = P.apply(B0) - A0, Q1 = P.apply(B1) - A0, Q2 = P.apply(B2) - A0;
  const f3 p1 = mk3(0, 0, 0), p2 = A1 - A0, p3 = A2 - A0;
  const f3 e1 = p2 - p1, e2 = p3 - p2, e3 = p1 - p3, f1 = Q1 - Q0, f2 = Q2 - Q1, f3v = Q0 - Q2;
  f3 ax[17];
  tri_axes(e1, e2, e3, f1, f2, f3v, ax, [](f3 x, f3 y) { return cross(x, y); });
  auto n1 = [](f3 v) { return fabsf(v.x) + fabsf(v.y) + fabsf(v.z); };
  const float le1 = n1(e1), le2 = n1(e2), le3 = n1(e3), lf1 = n1(f1), lf2 = n1(f2), lf3 = n1(f3v);
  const float ln = le1 * le2, lm = lf1 * lf2;
  const float bound[17] = {ln, lm, le1 * lf1, le1 * lf2, le1 * lf3, le2 * lf1, le2 * lf2, le2 * lf3,
                           le3 * lf1, le3 * lf2, le3 * lf3, le1 * ln, le2 * ln, le3 * ln, lf1 * lm, lf2 * lm,
                           lf3 * lm};
  // coordinate scale: the six points relative to A0 and the magnitudes the
  // pose arithmetic rounded
  float scale = n1(P.t) + n1(A0) + n1(B0);
  const f3 pts[5] = {p2, p3, Q0, Q1, Q2};
#pragma unroll
  for (int i = 0; i < 5; ++i) scale = fmaxf(scale, n1(pts[i]));
  bool ambiguous = false;
#pragma unroll
  for (int i = 0; i < 17; ++i) {
    const float P2v = dot(ax[i], p2), P3v = dot(ax[i], p3);
    const float Q1v = dot(ax[i], Q0), Q2v = dot(ax[i], Q1), Q3v = dot(ax[i], Q2);
    const float mn1 = fminf(0.f, fminf(P2v, P3v)), mx1 = fmaxf(0.f, fmaxf(P2v, P3v));
    const float mn2 = fminf(Q1v, fminf(Q2v, Q3v)), mx2 = fmaxf(Q1v, fmaxf(Q2v, Q3v));
    const float tol = 8e-6f * bound[i] * scale;
    const float g1 = mn1 - mx2, g2 = mn2 - mx1;
    if (g1 > tol || g2 > tol) return false;      // clearly separated along this axis
    if (g1 > -tol || g2 > -tol) ambiguous = true;  // within rounding of the threshold
  }
  return ambiguous ? tri_tri_fp64(P, A0, A1, A2, B0, B1, B2) : true;
}

}  // namespace

__global__ void __launch_bounds__(kMeshWarps * 32) mesh_collide_kernel(MeshArgs m) {
  __shared__ MeshSmem smem_all[kMeshWarps];
  MeshSmem& S = smem_all[threadIdx.x >> 5];
  const unsigned lane = threadIdx.x & 31u;
  const uint32_t gw = blockIdx.x * kMeshWarps + (threadIdx.x >> 5);
  const uint32_t nw = gridDim.x * kMeshWarps;
  for (uint32_t pose_i = gw; pose_i < m.n_poses; pose_i += nw) {
    Pose P;
    {
      const float4 q0 = __ldg(m.poses + 3 * (size_t)pose_i);
      const float4 q1 = __ldg(m.poses + 3 * (size_t)pose_i + 1);
      const float4 q2 = __ldg(m.poses + 3 * (size_t)pose_i + 2);
      P.r[0] = q0.x; P.r[1] = q0.y; P.r[2] = q0.z; P.r[3] = q0.w;
      P.r[4] = q1.x; P.r[5] = q1.y; P.r[6] = q1.z; P.r[7] = q1.w;
      P.r[8] = q2.x;
      P.t = mk3(q2.y, q2.z, q2.w);
    }
    if (lane == 0) {
      S.na[0] = 0;
      S.nb[0] = 0;
      S.found = 0;
    }
    int size = 1;
    uint32_t status = 0;
    __syncwarp();
    int found = 0;
    for (int round = 0; size > 0 && found < (int)m.max_contacts; ++round) {
      if (round >= kMaxRounds) { status |= 2u; break; }
      int k = size < 32 ? size : 32;
      if (k > kMeshStack - size) k = kMeshStack - size;  // room for two children per popped pair
      if (k <= 0) { status |= 1u; break; }
      uint32_t ia = 0, ib = 0;
      const bool active = (int)lane < k;
      if (active) {
        ia = S.na[size - 1 - lane];
        ib = S.nb[size - 1 - lane];
      }
      size -= k;
      __syncwarp();
      int push = 0;
      bool hit = false, down_a = false;
      uint32_t ca = 0, cb = 0;
      if (active && ia < m.a.n_nodes && ib < m.b.n_nodes) {
        const Node A = load_node(m.a.nodes, ia);
        const Node B = load_node(m.b.nodes, ib);
        if (obb_overlap(P, A, B)) {
          const bool la = A.child < 0, lb = B.child < 0;
          if (la && lb) {
            const uint32_t ta = (uint32_t)(-(A.child + 1)), tb = (uint32_t)(-(B.child + 1));
            if (ta < m.a.n_tris && tb < m.b.n_tris) {
              hit = tri_tri(P, ldv(m.a.tris, ta, 0), ldv(m.a.tris, ta, 1), ldv(m.a.tris, ta, 2), ldv(m.b.tris, tb, 0),
                            ldv(m.b.tris, tb, 1), ldv(m.b.tris, tb, 2));
              ca = ta;
              cb = tb;
            }
          } else {
            down_a = lb || (!la && sqn(A.e) > sqn(B.e));
            push = 2;
            ca = down_a ? (uint32_t)A.child : ia;
            cb = down_a ? ib : (uint32_t)B.child;
          }
        }
      }
      // push the two children of each descending pair (prefix sum over lanes)
      int incl = push;
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        const int t = __shfl_up_sync(0xFFFFFFFFu, incl, off);
        if ((int)lane >= off) incl += t;
      }
      const int total = __shfl_sync(0xFFFFFFFFu, incl, 31);
      if (push) {
        const int o = size + incl - push;
        S.na[o] = ca;
        S.nb[o] = cb;
        S.na[o + 1] = down_a ? ca + 1 : ca;
        S.nb[o + 1] = down_a ? cb : cb + 1;
      }
      size += total;
      // record contacts in lane order
      const unsigned hm = __ballot_sync(0xFFFFFFFFu, hit);
      if (hit) {
        const int slot = found + __popc(hm & ((1u << lane) - 1u));
        if (slot < (int)m.max_contacts) {
          m.pairs[((size_t)pose_i * m.max_contacts + slot) * 2 + 0] = (int32_t)ca;
          m.pairs[((size_t)pose_i * m.max_contacts + slot) * 2 + 1] = (int32_t)cb;
        }
      }
      found += __popc(hm);
      __syncwarp();
    }
    if (lane == 0) {
      const uint32_t cnt = found < (int)m.max_contacts ? (uint32_t)found : m.max_contacts;
      m.counts[pose_i] = cnt;
      m.flags[pose_i] = cnt > 0 ? 1 : 0;
      if (m.status) m.status[pose_i] = status;
    }
    __syncwarp();
  }
}

cudaError_t launch_mesh_collide(const MeshArgs& m, int blocks, cudaStream_t st) {
  if (m.n_poses == 0) return cudaSuccess;
  mesh_collide_kernel<<<blocks, kMeshWarps * 32, 0, st>>>(m);
  return cudaGetLastError();
}

}  // namespace fclg
