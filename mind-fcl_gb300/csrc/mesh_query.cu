// OBB BVH vs OBB BVH boolean collision of two triangle meshes for a batch of
// relative poses: one warp per pose, contacts in the reference's order.
//
// Restates OrientedNodeBVHSolver::MeshIntersect
// (narrowphase/detail/traversal/collision/bvh_solver-inl.h:74-164) with the
// penetration request off: node pairs whose boxes overlap (OBB overlap,
// math/bv/OBB-inl.h:305-436) descend into the node with the larger box
// (|extent|^2, OBB-inl.h:153-156; the FP64 value of the reference's own tree),
// leaf pairs run the 17-axis triangle test (intersect-inl.h:723-795, project6
// :1082-1102), and a pose keeps the first max_contacts colliding pairs
// (CollisionResult::addContact / terminationConditionSatisfied).
//
// Order.  The reference pops its stack depth first and, after descending,
// visits the second child (child + 1) before the first; a capped request
// reports the first max_contacts colliding leaf pairs of that order.  Here
// every pending node pair carries its path key: the descent choices from the
// root, one bit per step (0 = the child visited first), left-aligned above a
// sentinel bit.  Two keys compare as unsigned integers exactly as their
// places in the reference's visiting order.  The warp keeps its stack sorted
// (top = earliest), pops up to 32 node pairs per round, one per lane, and
// pushes each lane's children back above the entries that follow it, so the
// stack stays sorted.  Colliding leaf pairs go to a per-warp buffer with
// their keys; once it holds max_contacts of them, node pairs ordered after
// the last kept contact are dropped, and the pose ends when the earliest
// pending pair comes after it.  The kept contacts are written sorted by key:
// the reference's contact list.
//
// Arithmetic.  Box tests run in FP32 on boxes that contain their triangles,
// with a slack covering FP32 rounding, so they never drop a node pair whose
// subtree holds a colliding pair (extra node pairs visited change neither the
// contacts nor their keys).  The triangle test runs in FP32 and is re-decided
// in FP64, with each operation rounded as the reference's (no contraction),
// whenever an axis sits within its rounding bound of the separation
// threshold, so every verdict equals the reference's FP64 one.
#include "kernels.h"
#include "mesh_common.cuh"
#include "mesh_kernels.h"

namespace fclg {

namespace {

constexpr int kMeshStack = 512;
constexpr int kPathRoom = 64;           // slots kept for a depth-first descent (path length <= 62)
constexpr int kMeshWarps = 4;
constexpr int kSmemContacts = 128;      // in-shared-memory contact buffer (max_contacts <= 96)
constexpr int kMaxRounds = 1 << 22;     // bound against a corrupted tree

struct MeshSmem {
  uint32_t na[kMeshStack];
  uint32_t nb[kMeshStack];
  unsigned long long key[kMeshStack];
  unsigned long long ckey[kSmemContacts];
  int2 cpair[kSmemContacts];
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

// FP64 arithmetic rounded operation by operation (no fused multiply-add), the
// evaluation order of the reference's FP64 code.
__device__ __forceinline__ double mulr(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double addr(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double subr(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ d3 subr3(d3 a, d3 b) { return d3{subr(a.x, b.x), subr(a.y, b.y), subr(a.z, b.z)}; }
__device__ __forceinline__ double dotr(d3 a, d3 b) { return addr(addr(mulr(a.x, b.x), mulr(a.y, b.y)), mulr(a.z, b.z)); }
__device__ __forceinline__ d3 crossr(d3 a, d3 b) {
  return d3{subr(mulr(a.y, b.z), mulr(a.z, b.y)), subr(mulr(a.z, b.x), mulr(a.x, b.z)),
            subr(mulr(a.x, b.y), mulr(a.y, b.x))};
}

// FP64 triangle test, the reference's arithmetic (Q posed by the pose, every
// point taken relative to P1; intersect-inl.h:593-613, 723-795).
__device__ bool tri_tri_fp64(const Pose& P, f3 A0, f3 A1, f3 A2, f3 B0, f3 B1, f3 B2) {
  double R[9];
  for (int i = 0; i < 9; ++i) R[i] = P.r[i];
  const d3 T = tod(P.t);
  auto xf = [&](f3 qf) {
    const d3 q = tod(qf);
    return d3{addr(addr(addr(mulr(R[0], q.x), mulr(R[1], q.y)), mulr(R[2], q.z)), T.x),
              addr(addr(addr(mulr(R[3], q.x), mulr(R[4], q.y)), mulr(R[5], q.z)), T.y),
              addr(addr(addr(mulr(R[6], q.x), mulr(R[7], q.y)), mulr(R[8], q.z)), T.z)};
  };
  const d3 P1 = tod(A0);
  const d3 p1 = subr3(P1, P1), p2 = subr3(tod(A1), P1), p3 = subr3(tod(A2), P1);
  const d3 q1 = subr3(xf(B0), P1), q2 = subr3(xf(B1), P1), q3 = subr3(xf(B2), P1);
  d3 ax[17];
  tri_axes(subr3(p2, p1), subr3(p3, p2), subr3(p1, p3), subr3(q2, q1), subr3(q3, q2), subr3(q1, q3), ax,
           [](d3 x, d3 y) { return crossr(x, y); });
  for (int i = 0; i < 17; ++i) {
    const double P1v = dotr(ax[i], p1), P2v = dotr(ax[i], p2), P3v = dotr(ax[i], p3);
    const double Q1v = dotr(ax[i], q1), Q2v = dotr(ax[i], q2), Q3v = dotr(ax[i], q3);
    const double mn1 = fmin(P1v, fmin(P2v, P3v)), mx2 = fmax(Q1v, fmax(Q2v, Q3v));
    if (mn1 > mx2) return false;
    const double mx1 = fmax(P1v, fmax(P2v, P3v)), mn2 = fmin(Q1v, fmin(Q2v, Q3v));
    if (mn2 > mx1) return false;
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

// CTAs per SM the kernel's register budget is sized for: four (128
// registers, a few spilled) beat the three that 138 registers allow
// (measured: first contact 4.40 -> 4.65 M collides/s).
#ifndef FCLG_MESH_MINB
#define FCLG_MESH_MINB 4
#endif

__global__ void __launch_bounds__(kMeshWarps * 32, FCLG_MESH_MINB) mesh_collide_kernel(MeshArgs m) {
  __shared__ MeshSmem smem_all[kMeshWarps];
  MeshSmem& S = smem_all[threadIdx.x >> 5];
  const unsigned lane = threadIdx.x & 31u;
  const uint32_t gw = blockIdx.x * kMeshWarps + (threadIdx.x >> 5);
  const uint32_t nw = gridDim.x * kMeshWarps;
  const int cap = (int)m.max_contacts;
  // contact buffer: max_contacts + 32 entries (one round's hits past a full
  // buffer), rounded up to a power of two for the sort
  const int cbuf = pow2_at_least(cap + 32);
  unsigned long long* ckey = S.ckey;
  int2* cpair = S.cpair;
  uint32_t n_box = 0, n_leaf = 0;  // this lane's tests (traffic counters)
  if (cbuf > kSmemContacts) {
    ckey = m.cbuf_key + (size_t)gw * m.cbuf_len;
    cpair = m.cbuf_pair + (size_t)gw * m.cbuf_len;
  }
  // poses differ in traversal work by orders of magnitude: with m.next each
  // warp takes its next pose as it finishes one
  auto take = [&](uint32_t done) -> uint32_t {
    if (!m.next) return done + nw;
    uint32_t k = 0;
    if (lane == 0) k = atomicAdd(m.next, 1u);
    return __shfl_sync(0xFFFFFFFFu, k, 0);
  };
  for (uint32_t pose_i = m.next ? take(0) : gw; pose_i < m.n_poses; pose_i = take(pose_i)) {
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
      S.key[0] = kRootKey;
    }
    int size = 1;
    uint32_t status = 0;
    int found = 0;                    // contacts in the buffer
    unsigned long long last = kNoKey;  // key of the max_contacts-th kept contact once the buffer is full
    __syncwarp();
    for (int round = 0; size > 0; ++round) {
      if (round >= kMaxRounds) { status |= 2u; break; }
      // the earliest pending pair comes after every kept contact: done
      if (found >= cap && S.key[size - 1] > last) break;
      // Up to 32 pairs per round while the stack keeps kPathRoom free slots,
      // one pair per round (plain depth-first) above that: from any state a
      // depth-first descent needs at most one slot per level of the path
      // (<= 62, checked on the host), so the stack never overflows.
      int k = size < 32 ? size : 32;
      const int room = kMeshStack - kPathRoom - size;
      if (k > room) k = room > 1 ? room : 1;
      if (size + k > kMeshStack) { status |= 1u; break; }  // unreachable by the bound above
      uint32_t ia = 0, ib = 0;
      unsigned long long key = kNoKey;
      const bool popped = (int)lane < k;
      if (popped) {
        ia = S.na[size - 1 - lane];
        ib = S.nb[size - 1 - lane];
        key = S.key[size - 1 - lane];
      }
      size -= k;
      __syncwarp();
      int push = 0;
      bool hit = false, down_a = false;
      uint32_t ca = 0, cb = 0;
      if (popped && key < last && ia < m.a.n_nodes && ib < m.b.n_nodes) {
        const Node A = load_node(m.a.nodes, ia);
        const Node B = load_node(m.b.nodes, ib);
        ++n_box;
        if (obb_overlap(P, A, B)) {
          const bool la = A.child < 0, lb = B.child < 0;
          if (la && lb) {
            const uint32_t ta = (uint32_t)(-(A.child + 1)), tb = (uint32_t)(-(B.child + 1));
            if (ta < m.a.n_tris && tb < m.b.n_tris) {
              ++n_leaf;
              hit = tri_tri(P, ldv(m.a.tris, ta, 0), ldv(m.a.tris, ta, 1), ldv(m.a.tris, ta, 2), ldv(m.b.tris, tb, 0),
                            ldv(m.b.tris, tb, 1), ldv(m.b.tris, tb, 2));
              ca = ta;
              cb = tb;
            }
          } else if ((key & 1ull) == 0ull) {
            down_a = lb || (!la && __ldg(m.a.size + ia) > __ldg(m.b.size + ib));
            push = 2;
            ca = down_a ? (uint32_t)A.child : ia;
            cb = down_a ? ib : (uint32_t)B.child;
          } else {
            status |= 4u;  // path longer than the key holds (rejected on the host)
          }
        }
      }
      // Children go back above the entries that follow their parent: lane j's
      // pair lands below those of lanes < j.  Exclusive suffix sum over lanes.
      // (every push is two entries: the suffix sum is twice a population count)
      const unsigned pm = __ballot_sync(0xFFFFFFFFu, push != 0);
      const int incl = 2 * __popc(pm >> lane);
      const int total = 2 * __popc(pm);
      if (push) {
        const int o = size + incl - push;  // slots o (visited later), o + 1 (visited first)
        S.na[o + 1] = down_a ? ca + 1 : ca;
        S.nb[o + 1] = down_a ? cb : cb + 1;
        S.key[o + 1] = child_key(key, 0);
        S.na[o] = ca;
        S.nb[o] = cb;
        S.key[o] = child_key(key, 1);
      }
      size += total;
      // colliding leaf pairs into the buffer (lane order = key order)
      const unsigned hm = __ballot_sync(0xFFFFFFFFu, hit);
      if (hit) {
        const int slot = found + __popc(hm & ((1u << lane) - 1u));
        ckey[slot] = key;
        cpair[slot] = make_int2((int)ca, (int)cb);
      }
      found += __popc(hm);
      __syncwarp();
      if (hm) last = keep_first(ckey, cpair, found, cap, lane, last);  // keep the max_contacts earliest
    }
    sort_found(ckey, cpair, found, cap, lane);
    for (int i = (int)lane; i < found; i += 32) {
      const int2 p = cpair[i];
      m.pairs[((size_t)pose_i * m.max_contacts + i) * 2 + 0] = p.x;
      m.pairs[((size_t)pose_i * m.max_contacts + i) * 2 + 1] = p.y;
    }
    if (lane == 0) {
      m.counts[pose_i] = (uint32_t)found;
      m.flags[pose_i] = found > 0 ? 1 : 0;
      if (m.status) m.status[pose_i] = status;
    }
    __syncwarp();
  }
  if (m.counters) {
    unsigned long long a = n_box, b = n_leaf;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      a += __shfl_down_sync(0xFFFFFFFFu, a, off);
      b += __shfl_down_sync(0xFFFFFFFFu, b, off);
    }
    if (lane == 0) {
      atomicAdd(m.counters, a);
      atomicAdd(m.counters + 1, b);
    }
  }
}

int mesh_contact_buffer_len(uint32_t max_contacts) {
  int p = 2;
  while (p < (int)max_contacts + 32) p <<= 1;
  return p > kSmemContacts ? p : 0;
}

int mesh_collide_warps(int blocks) { return blocks * kMeshWarps; }

int mesh_collide_resident_blocks(int num_sms) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mesh_collide_kernel, kMeshWarps * 32, 0) != cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  return num_sms * per_sm;
}

cudaError_t launch_mesh_collide(const MeshArgs& m, int blocks, cudaStream_t st) {
  if (m.n_poses == 0) return cudaSuccess;
  mesh_collide_kernel<<<blocks, kMeshWarps * 32, 0, st>>>(m);
  return cudaGetLastError();
}

}  // namespace fclg
