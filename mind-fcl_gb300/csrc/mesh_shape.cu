// fcl::collide of a triangle mesh (OBB tree) against a shape, penetration off,
// for a batch of (shape, pose) queries: one warp per query.
//
// Restates OrientedNodeBVHSolver::MeshShapeIntersect
// (narrowphase/detail/traversal/collision/bvh_solver-inl.h:6-72): the shape's
// bounding box against the tree's boxes (OBB overlap, math/bv/OBB-inl.h:
// 305-436), and at the leaves the shape-triangle test fcl::collide picks
// (GJKSolver::shapeTriangleIntersect with the triangle's transform,
// gjk_solver-inl.h:451-591): sphereTriangleIntersect
// (sphere_triangle-inl.h:52-191) for spheres, boxTriangleIntersect
// (box_triangle-inl.h) for boxes, MPR::Intersect on (shape, triangle) for the
// rest.  A query stops once it has max_contacts colliding triangles.
//
// GPU layout: as the mesh-mesh kernel -- node ids with their path keys on a
// per-warp stack in shared memory kept in the reference's visiting order (the
// second child first), up to 32 popped per round (one per lane) while 64
// slots stay free, children pushed back above the entries that follow their
// parent; colliding triangles go to a per-warp buffer with their keys and the
// first max_contacts of the reference's order are kept and written in that
// order.  The shape's box is built once per query (a hull's extent by a warp
// reduction over its vertices).  The sphere and box leaf tests run in FP32 and are re-decided in
// FP64 when a comparison sits within its rounding bound, so their verdicts
// equal the FP64 ones; the MPR leaves run in FP32.
#include "gjk.cuh"
#include "kernels.h"
#include "mesh_common.cuh"
#include "mesh_kernels.h"
#include "mpr.cuh"
#include "support.cuh"

namespace fclg {

namespace {

constexpr int kMsStack = 512;
constexpr int kMsPathRoom = 64;     // slots kept for a depth-first descent (path length <= 62)
constexpr int kMsSmemContacts = 128;  // in-shared-memory contact buffer (max_contacts <= 96)
constexpr int kMsWarps = 4;
// CTAs per SM the kernel is compiled for (its register budget)
#ifndef FCLG_MESH_SHAPE_MINB
#define FCLG_MESH_SHAPE_MINB 4
#endif
constexpr int kMsMaxRounds = 1 << 22;  // bound against a corrupted tree

struct MsSmem {
  uint32_t node[kMsStack];
  unsigned long long key[kMsStack];
  unsigned long long ckey[kMsSmemContacts];
  int2 cval[kMsSmemContacts];
};

struct D3 {
  double x, y, z;
};
__device__ __forceinline__ D3 dd(f3 v) { return D3{v.x, v.y, v.z}; }
__device__ __forceinline__ D3 operator-(D3 a, D3 b) { return D3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ D3 operator*(D3 a, double s) { return D3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ double ddot(D3 a, D3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ D3 dcross(D3 a, D3 b) {
  return D3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// sphere_triangle-inl.h:52-78
__device__ double seg_sqr_dist64(D3 from, D3 to, D3 p) {
  D3 diff = p - from;
  const D3 v = to - from;
  double t = ddot(v, diff);
  if (t > 0) {
    const double vv = ddot(v, v);
    if (t < vv) diff = diff - v * (t / vv);
    else diff = diff - v;
  }
  return ddot(diff, diff);
}

// sphereTriangleIntersect, sphere_triangle-inl.h:107-191, the boolean in FP64
__device__ __noinline__ bool sphere_tri64(double r, D3 c, D3 P1, D3 P2, D3 P3) {
  D3 n = dcross(P2 - P1, P3 - P1);
  const double nl = sqrt(ddot(n, n));
  if (nl > 0) n = n * (1.0 / nl);
  const double rt = r + 2.220446049250313e-16;
  double dist = ddot(c - P1, n);
  if (dist < 0) {
    dist = -dist;
    n = n * -1.0;
  }
  if (!(dist < rt)) return false;
  const double r1 = ddot(dcross(P2 - P1, n), c - P1), r2 = ddot(dcross(P3 - P2, n), c - P2),
               r3 = ddot(dcross(P1 - P3, n), c - P3);
  if ((r1 > 0 && r2 > 0 && r3 > 0) || (r1 <= 0 && r2 <= 0 && r3 <= 0)) return true;  // contact at distance `dist`
  const double rr = rt * rt;
  return seg_sqr_dist64(P1, P2, c) < rr || seg_sqr_dist64(P2, P3, c) < rr || seg_sqr_dist64(P3, P1, c) < rr;
}

// The same test in FP32: 1 hit, 0 miss, -1 within rounding of the radius.
__device__ __forceinline__ int sphere_tri32(float r, f3 c, f3 P1, f3 P2, f3 P3) {
  const f3 n = normalized(cross(P2 - P1, P3 - P1));
  const float scale = 1.f + fmaxf(fmaxf(fabsf(c.x), fabsf(c.y)), fabsf(c.z)) +
                      fmaxf(fmaxf(absnorm(P1), absnorm(P2)), absnorm(P3));
  const float m = 8e-6f * scale;
  const float dist = fabsf(dot(c - P1, n));
  float d;
  const f3 nn = dot(c - P1, n) < 0.f ? -n : n;
  const float r1 = dot(cross(P2 - P1, nn), c - P1), r2 = dot(cross(P3 - P2, nn), c - P2),
              r3 = dot(cross(P1 - P3, nn), c - P3);
  const float rm = m * scale;
  const bool in = (r1 > rm && r2 > rm && r3 > rm) || (r1 < -rm && r2 < -rm && r3 < -rm);
  const bool out = (r1 < -rm || r2 < -rm || r3 < -rm) && (r1 > rm || r2 > rm || r3 > rm);
  if (in) {
    d = dist;
  } else {
    auto seg = [](f3 a, f3 b, f3 p) {
      const f3 v = b - a;
      f3 diff = p - a;
      const float t = dot(v, diff);
      if (t > 0.f) {
        const float vv = dot(v, v);
        diff = t < vv ? diff - v * (t / vv) : diff - v;
      }
      return dot(diff, diff);
    };
    const float e2 = fminf(seg(P1, P2, c), fminf(seg(P2, P3, c), seg(P3, P1, c)));
    d = sqrtf(e2);
    if (!out) d = fminf(d, dist);  // the face may hold the closest point: decide in FP64 below if near
    if (!out && fabsf(d - r) <= m) return -1;
  }
  if (d < r - m) return 1;
  if (d > r + m) return 0;
  return -1;
}

// box_triangle-inl.h:9-69 in FP64 (triangle in the box's frame, h half sides)
__device__ bool box_tri_edge64(D3 h, D3 e, D3 v0, D3 v1) {
  const double ax = fabs(e.x), ay = fabs(e.y), az = fabs(e.z);
  auto sep = [](double r, double p0, double p1) { return p0 < p1 ? (p0 > r || p1 < -r) : (p1 > r || p0 < -r); };
  if (sep(h.y * az + h.z * ay, v0.y * e.z - v0.z * e.y, v1.y * e.z - v1.z * e.y)) return true;
  if (sep(h.x * az + h.z * ax, v0.x * e.z - v0.z * e.x, v1.x * e.z - v1.z * e.x)) return true;
  if (sep(h.x * ay + h.y * ax, v0.x * e.y - v0.y * e.x, v1.x * e.y - v1.y * e.x)) return true;
  return false;
}

// detectBoxTriangleOverlap, box_triangle-inl.h:71-119, in FP64
__device__ __noinline__ bool box_tri64(D3 h, D3 v0, D3 v1, D3 v2) {
  const double hv[3] = {h.x, h.y, h.z};
  const double a[3] = {v0.x, v0.y, v0.z}, b[3] = {v1.x, v1.y, v1.z}, c[3] = {v2.x, v2.y, v2.z};
  for (int i = 0; i < 3; ++i) {
    const double mn = fmin(a[i], fmin(b[i], c[i])), mx = fmax(a[i], fmax(b[i], c[i]));
    if (mx < -hv[i] || mn > hv[i]) return false;
  }
  const D3 e0 = v1 - v0, e1 = v2 - v1, e2 = v0 - v2;
  if (box_tri_edge64(h, e0, v0, v2) || box_tri_edge64(h, e1, v1, v0) || box_tri_edge64(h, e2, v0, v1)) return false;
  const D3 n = dcross(e0, e1);
  const double nv[3] = {n.x, n.y, n.z};
  double pmin[3], pmax[3];
  for (int i = 0; i < 3; ++i) {
    if (nv[i] > 0) {
      pmin[i] = -hv[i] - a[i];
      pmax[i] = hv[i] - a[i];
    } else {
      pmin[i] = hv[i] - a[i];
      pmax[i] = -hv[i] - a[i];
    }
  }
  return ((nv[0] * pmin[0] + nv[1] * pmin[1]) + nv[2] * pmin[2]) <= 0 &&
         ((nv[0] * pmax[0] + nv[1] * pmax[1]) + nv[2] * pmax[2]) >= 0;
}

// The same test in FP32: 1 overlap, 0 separated, -1 a comparison within rounding.
__device__ __forceinline__ int box_tri32(f3 h, f3 v0, f3 v1, f3 v2) {
  const float scale = 1.f + fmaxf(absnorm(h), fmaxf(absnorm(v0), fmaxf(absnorm(v1), absnorm(v2))));
  const float m1 = 4e-6f * scale, m2 = 1.6e-5f * scale * scale, m3 = 4e-5f * scale * scale * scale;
  bool amb = false;
  // "x > r" with a margin: 1 true, 0 false, ambiguous flagged
  auto gt = [&](float x, float r, float m) {
    if (x > r + m) return true;
    if (x >= r - m) amb = true;
    return false;
  };
  const float hv[3] = {h.x, h.y, h.z};
  const float a[3] = {v0.x, v0.y, v0.z}, b[3] = {v1.x, v1.y, v1.z}, c[3] = {v2.x, v2.y, v2.z};
  for (int i = 0; i < 3; ++i) {
    const float mn = fminf(a[i], fminf(b[i], c[i])), mx = fmaxf(a[i], fmaxf(b[i], c[i]));
    if (gt(-hv[i], mx, m1) || gt(mn, hv[i], m1)) return 0;
  }
  auto edge = [&](f3 e, f3 p0, f3 p1) {
    const float ax = fabsf(e.x), ay = fabsf(e.y), az = fabsf(e.z);
    auto sep = [&](float r, float q0, float q1) {
      const float lo = fminf(q0, q1), hi = fmaxf(q0, q1);
      return gt(lo, r, m2) || gt(-hi, r, m2);
    };
    return sep(h.y * az + h.z * ay, p0.y * e.z - p0.z * e.y, p1.y * e.z - p1.z * e.y) ||
           sep(h.x * az + h.z * ax, p0.x * e.z - p0.z * e.x, p1.x * e.z - p1.z * e.x) ||
           sep(h.x * ay + h.y * ax, p0.x * e.y - p0.y * e.x, p1.x * e.y - p1.y * e.x);
  };
  const f3 e0 = v1 - v0, e1 = v2 - v1, e2 = v0 - v2;
  if (edge(e0, v0, v2) || edge(e1, v1, v0) || edge(e2, v0, v1)) return 0;
  const f3 n = cross(e0, e1);
  const float nv[3] = {n.x, n.y, n.z};
  float smin = 0.f, smax = 0.f;
  for (int i = 0; i < 3; ++i) {
    const float lo = nv[i] > 0.f ? -hv[i] - a[i] : hv[i] - a[i];
    const float hi = nv[i] > 0.f ? hv[i] - a[i] : -hv[i] - a[i];
    smin = fmaf(nv[i], lo, smin);
    smax = fmaf(nv[i], hi, smax);
    if (fabsf(nv[i]) <= m2) amb = true;  // the sign choice itself is near its threshold
  }
  if (gt(smin, 0.f, m3) || gt(0.f, smax, m3)) return 0;
  return amb ? -1 : 1;
}

// The shape's own-axes bounding box (centre and half sides in its frame), as
// computeBV builds an OBB (geometry/shape/utility-inl.h:93-219, 780-789): box
// half sides; sphere radius on the mesh's axes; capsule (r, r, lz/2 + r);
// cylinder (r, r, lz/2); a hull its vertices' extent (the reference fits
// principal axes; any box that bounds the shape prunes the same leaves).
__device__ void shape_box(const ShapeDev& s, const float4* __restrict__ verts, unsigned lane, f3& c, f3& e,
                          bool& own_axes) {
  own_axes = true;
  c = mk3(0.f, 0.f, 0.f);
  switch (s.type) {
    case kBox: e = mk3(s.p0, s.p1, s.p2); break;
    case kSphere: e = mk3(s.p0, s.p0, s.p0); own_axes = false; break;
    case kCapsule: e = mk3(s.p0, s.p0, s.p1 + s.p0); break;
    case kCylinder: e = mk3(s.p0, s.p0, s.p1); break;
    default: {
      f3 lo = mk3(INFINITY, INFINITY, INFINITY), hi = mk3(-INFINITY, -INFINITY, -INFINITY);
      for (uint32_t i = lane; i < s.nv; i += 32) {
        const float4 q = __ldg(verts + s.vofs + i);
        lo = mk3(fminf(lo.x, q.x), fminf(lo.y, q.y), fminf(lo.z, q.z));
        hi = mk3(fmaxf(hi.x, q.x), fmaxf(hi.y, q.y), fmaxf(hi.z, q.z));
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        lo.x = fminf(lo.x, __shfl_xor_sync(0xFFFFFFFFu, lo.x, off));
        lo.y = fminf(lo.y, __shfl_xor_sync(0xFFFFFFFFu, lo.y, off));
        lo.z = fminf(lo.z, __shfl_xor_sync(0xFFFFFFFFu, lo.z, off));
        hi.x = fmaxf(hi.x, __shfl_xor_sync(0xFFFFFFFFu, hi.x, off));
        hi.y = fmaxf(hi.y, __shfl_xor_sync(0xFFFFFFFFu, hi.y, off));
        hi.z = fmaxf(hi.z, __shfl_xor_sync(0xFFFFFFFFu, hi.z, off));
      }
      c = (lo + hi) * 0.5f;
      e = (hi - lo) * 0.5f;
    }
  }
}

}  // namespace

template <bool PEN>
__global__ void __launch_bounds__(kMsWarps * 32, FCLG_MESH_SHAPE_MINB) mesh_shape_kernel(MeshShapeArgs m) {
  __shared__ MsSmem smem_all[kMsWarps];
  MsSmem& S = smem_all[threadIdx.x >> 5];
  const unsigned lane = threadIdx.x & 31u;
  const uint32_t gw = blockIdx.x * kMsWarps + (threadIdx.x >> 5);
  const uint32_t nw = gridDim.x * kMsWarps;
  const int cap = (int)m.max_contacts;
  unsigned long long* ckey = S.ckey;
  int2* cval = S.cval;
  if (pow2_at_least(cap + 32) > kMsSmemContacts) {
    ckey = m.cbuf_key + (size_t)gw * m.cbuf_len;
    cval = m.cbuf_val + (size_t)gw * m.cbuf_len;
  }
  // with m.next each warp takes its next query as it finishes one
  auto take = [&](uint32_t done) -> uint32_t {
    if (!m.next) return done + nw;
    uint32_t k = 0;
    if (lane == 0) k = atomicAdd(m.next, 1u);
    return __shfl_sync(0xFFFFFFFFu, k, 0);
  };
  for (uint32_t q = m.next ? take(0) : gw; q < m.n; q = take(q)) {
    Pose X;  // the shape in the mesh frame
    {
      const float4 q0 = __ldg(m.poses + 3 * (size_t)q);
      const float4 q1 = __ldg(m.poses + 3 * (size_t)q + 1);
      const float4 q2 = __ldg(m.poses + 3 * (size_t)q + 2);
      X.r[0] = q0.x; X.r[1] = q0.y; X.r[2] = q0.z; X.r[3] = q0.w;
      X.r[4] = q1.x; X.r[5] = q1.y; X.r[6] = q1.z; X.r[7] = q1.w;
      X.r[8] = q2.x;
      X.t = mk3(q2.y, q2.z, q2.w);
    }
    const uint32_t sid = __ldg(m.shape_ids + q);
    uint32_t status = 0;
    int found = 0;
    if (sid < m.n_shapes) {
      const ShapeDev shp = load_shape(m.shapes, sid);
      // the shape's box in the mesh frame, widened by the FP32 rounding of its placement
      f3 cl, e;
      bool own;
      shape_box(shp, m.verts, lane, cl, e, own);
      Node SB;
#pragma unroll
      for (int k = 0; k < 9; ++k) SB.a[k] = own ? X.r[k] : ((k % 4 == 0) ? 1.f : 0.f);
      SB.c = X.apply(cl);
      const float grow = 4e-6f * (1.f + absnorm(SB.c) + absnorm(e));
      SB.e = mk3(e.x + grow, e.y + grow, e.z + grow);
      SB.child = 0;
      Pose I;
#pragma unroll
      for (int k = 0; k < 9; ++k) I.r[k] = (k % 4 == 0) ? 1.f : 0.f;
      I.t = mk3(0.f, 0.f, 0.f);
      // the triangle in the shape's frame: X^-1
      Pose Xi;
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) Xi.r[3 * r + c] = X.r[3 * c + r];
      Xi.t = -Xi.rot(X.t);
      MinkowskiSupport<1> sup;
      sup.A = shp;
      sup.B.type = kTriangle;
      sup.B.nv = 3;
      sup.B.p0 = sup.B.p1 = sup.B.p2 = 0.f;
      sup.pose = Xi;
      sup.verts = m.verts;
      sup.hull = m.mesh.tris;
      sup.g = Group<1>::make();
      const f3 interior_a = load_interior(m.shapes, sid, shp.type);

      if (lane == 0) {
        S.node[0] = 0;
        S.key[0] = kRootKey;
      }
      int size = 1;
      unsigned long long last = kNoKey;  // key of the max_contacts-th kept contact once the buffer is full
      __syncwarp();
      for (int round = 0; size > 0; ++round) {
        if (round >= kMsMaxRounds) { status |= 2u; break; }
        // the earliest pending node comes after every kept contact: done
        if (found >= cap && S.key[size - 1] > last) break;
        int k = size < 32 ? size : 32;
        const int room = kMsStack - kMsPathRoom - size;
        if (k > room) k = room > 1 ? room : 1;
        if (size + k > kMsStack) { status |= 1u; break; }  // unreachable: a descent needs <= 62 slots
        const bool popped = (int)lane < k;
        uint32_t id = 0;
        unsigned long long key = kNoKey;
        if (popped) {
          id = S.node[size - 1 - lane];
          key = S.key[size - 1 - lane];
        }
        size -= k;
        __syncwarp();
        int push = 0;
        bool hit = false;
        uint32_t child = 0, tri = 0;
        if (popped && key < last && id < m.mesh.n_nodes) {
          const Node N = load_node(m.mesh.nodes, id);
          if (obb_overlap(I, SB, N)) {
            if (N.child >= 0) {
              if ((key & 1ull) == 0ull) {
                push = 2;
                child = (uint32_t)N.child;
              } else {
                status |= 8u;  // path longer than the key holds (rejected on the host)
              }
            } else {
              tri = (uint32_t)(-(N.child + 1));
              if (tri < m.mesh.n_tris) {
                const f3 P1 = ldv(m.mesh.tris, tri, 0), P2 = ldv(m.mesh.tris, tri, 1), P3 = ldv(m.mesh.tris, tri, 2);
                if (shp.type == kSphere) {
                  const int v = sphere_tri32(shp.p0, X.t, P1, P2, P3);
                  hit = v >= 0 ? v == 1 : sphere_tri64(shp.p0, dd(X.t), dd(P1), dd(P2), dd(P3));
                } else if (PEN) {
                  // with penetration the leaf is GJK's verdict, the test EPA starts from
                  // (shapeTriangleIntersectImplRun, gjk_solver-inl.h:335-341; the box's
                  // specialisation defers to it when a contact is wanted, :434-449)
                  MinkowskiSupport<1> s2 = sup;
                  s2.B.vofs = 3 * tri;
                  Simplex s0;
                  hit = gjk_evaluate(s2, mk3(-1.f, 0.f, 0.f), m.gjk_tol, m.gjk_max_iter, false, s0).status ==
                        kGjkIntersect;
                } else if (shp.type == kBox) {
                  const f3 w1 = Xi.apply(P1), w2 = Xi.apply(P2), w3 = Xi.apply(P3);
                  const int v = box_tri32(mk3(shp.p0, shp.p1, shp.p2), w1, w2, w3);
                  if (v >= 0) {
                    hit = v == 1;
                  } else {
                    // FP64 placement of the triangle in the box frame
                    D3 t64[3];
                    const f3 Ps[3] = {P1, P2, P3};
                    for (int j = 0; j < 3; ++j) {
                      const D3 dlt = dd(Ps[j]) - dd(X.t);
                      t64[j] = D3{((double)X.r[0] * dlt.x + (double)X.r[3] * dlt.y) + (double)X.r[6] * dlt.z,
                                  ((double)X.r[1] * dlt.x + (double)X.r[4] * dlt.y) + (double)X.r[7] * dlt.z,
                                  ((double)X.r[2] * dlt.x + (double)X.r[5] * dlt.y) + (double)X.r[8] * dlt.z};
                    }
                    hit = box_tri64(D3{shp.p0, shp.p1, shp.p2}, t64[0], t64[1], t64[2]);
                  }
                } else {
                  // MPR::Intersect on (shape, triangle) (use_mpr_if_no_contact, gjk_solver-inl.h:471-477)
                  MinkowskiSupport<1> s2 = sup;
                  s2.B.vofs = 3 * tri;
                  Mpr<MinkowskiSupport<1>> mpr{s2, m.gjk_max_iter, m.gjk_tol};
                  const f3 v0 = interior_a - Xi.apply((P1 + P2 + P3) * (1.f / 3.f));
                  hit = mpr.intersect(v0) == MprStatus::Intersect;
                }
              }
            }
          }
        }
        // Children go back above the entries that follow their parent (lane j's
        // below those of lanes < j), the second child on top: the reference
        // pushes the first child, then the second, and pops the second first.
        // (every push is two entries: the suffix sum is twice a population count)
        const unsigned pm = __ballot_sync(0xFFFFFFFFu, push != 0);
        const int incl = 2 * __popc(pm >> lane);
        const int total = 2 * __popc(pm);
        if (push) {
          const int o = size + incl - push;
          S.node[o + 1] = child + 1;
          S.key[o + 1] = child_key(key, 0);
          S.node[o] = child;
          S.key[o] = child_key(key, 1);
        }
        size += total;
        const unsigned hm = __ballot_sync(0xFFFFFFFFu, hit);
        if (hit) {
          const int slot = found + __popc(hm & ((1u << lane) - 1u));
          ckey[slot] = key;
          cval[slot] = make_int2((int)tri, 0);
        }
        found += __popc(hm);
        __syncwarp();
        if (hm) last = keep_first(ckey, cval, found, cap, lane, last);
      }
      sort_found(ckey, cval, found, cap, lane);
      for (int i = (int)lane; i < found; i += 32) m.tri_ids[(size_t)q * m.max_contacts + i] = cval[i].x;
      __syncwarp();
    }
    if (lane == 0) {
      const uint32_t cnt = (uint32_t)found;
      m.counts[q] = cnt;
      m.flags[q] = cnt > 0 ? 1 : 0;
      if (m.status) m.status[q] = status | (sid < m.n_shapes ? 0u : 4u);
    }
    __syncwarp();
  }
}

int mesh_shape_warps(int blocks) { return blocks * kMsWarps; }

int mesh_shape_resident_blocks(int num_sms, bool penetration) {
  int per_sm = 0;
  const cudaError_t e =
      penetration ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mesh_shape_kernel<true>, kMsWarps * 32, 0)
                  : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mesh_shape_kernel<false>, kMsWarps * 32, 0);
  if (e != cudaSuccess || per_sm < 1) per_sm = 1;
  return num_sms * per_sm;
}

cudaError_t launch_mesh_shape(const MeshShapeArgs& m, int blocks, cudaStream_t st) {
  if (m.n == 0) return cudaSuccess;
  if (m.contacts) mesh_shape_kernel<true><<<blocks, kMsWarps * 32, 0, st>>>(m);
  else mesh_shape_kernel<false><<<blocks, kMsWarps * 32, 0, st>>>(m);
  return cudaGetLastError();
}

}  // namespace fclg
