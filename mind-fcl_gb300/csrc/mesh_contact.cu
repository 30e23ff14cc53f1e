// Contacts of mesh-shape collisions with penetration on (fcl::collide of a
// BVHModel<OBBRSS> and a shape with a contact-requesting CollisionRequest):
// for every triangle the traversal reported, the contact of
// ShapePairIntersectSolver::ShapeSimplexIntersect
// (narrowphase/detail/shape_pair_intersect-inl.h:132-170) -- a sphere in
// closed form (sphereTriangleIntersect, primitive_shape_algorithm/
// sphere_triangle-inl.h:107-191, in FP64), every other shape by GJK then EPA
// on the shape and the triangle (shapeTriangleIntersectImplRun,
// gjk_solver-inl.h:305-375) -- with the normal reversed as the mesh-shape
// contact meta asks (bvh_solver-inl.h:56-61, shape_pair_intersect-inl.h:19-26).
// One warp per contact: lane 0 runs GJK, the warp runs EPA in the
// reference's 256-face layout in shared memory.
#include "epa.cuh"
#include "gjk.cuh"
#include "mesh_common.cuh"
#include "mesh_kernels.h"

namespace fclg {
namespace {

constexpr int kMcWarps = 4, kMcF = 256, kMcV = 192;

// Support of (shape, triangle) with the triangle posed in the shape's frame,
// the shape's support spread over the warp's lanes.
struct TriSupport32 {
  ShapeDev A;
  Pose pose;                  // the triangle's frame (the mesh) in the shape's frame
  const float4* __restrict__ verts;
  f3 t0, t1, t2;              // the triangle in the mesh frame
  Group<32> g;
  __device__ __forceinline__ void operator()(f3 d, f3& pa, f3& pb) const {
    pa = shape_support<32>(A, verts, d, g);
    // triangleSupport (geometry/shape/shape_gjk_interface-inl.h:17-39) along -R^T d
    const f3 e = pose.rotT(-d);
    const float da = dot(e, t0), db = dot(e, t1), dc = dot(e, t2);
    const f3 s = da > db ? (dc > da ? t2 : t0) : (dc > db ? t2 : t1);
    pb = pose.apply(s);
  }
};

__device__ __forceinline__ d3 dneg(d3 a) { return d3{-a.x, -a.y, -a.z}; }
__device__ __forceinline__ double dsq(d3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
__device__ __forceinline__ d3 dnormalized(d3 a) {  // Eigen's normalize(): a zero vector stays zero
  const double n2 = dsq(a);
  if (!(n2 > 0.0)) return a;
  return a * (1.0 / sqrt(n2));
}

// segmentSqrDistance (sphere_triangle-inl.h:52-78)
__device__ double seg_sqr(d3 from, d3 to, d3 p, d3& nearest) {
  d3 diff = p - from;
  const d3 v = to - from;
  double t = dot(v, diff);
  if (t > 0) {
    const double vv = dot(v, v);
    if (t < vv) {
      t /= vv;
      diff = diff - v * t;
    } else {
      t = 1;
      diff = diff - v;
    }
  } else {
    t = 0;
  }
  nearest = from + v * t;
  return dot(diff, diff);
}

// projectInTriangle (sphere_triangle-inl.h:81-104)
__device__ bool project_in(d3 p1, d3 p2, d3 p3, d3 n, d3 p) {
  const double r1 = dot(cross(p2 - p1, n), p - p1);
  const double r2 = dot(cross(p3 - p2, n), p - p2);
  const double r3 = dot(cross(p1 - p3, n), p - p3);
  return (r1 > 0 && r2 > 0 && r3 > 0) || (r1 <= 0 && r2 <= 0 && r3 <= 0);
}

// sphereTriangleIntersect with its contact (sphere_triangle-inl.h:107-191):
// contact point, normal from the centre towards it, and the reference's
// depth -(r - distance).
__device__ bool sphere_tri_contact(double r, d3 c, d3 P1, d3 P2, d3 P3, d3& pos, d3& normal, double& depth) {
  d3 n = dnormalized(cross(P2 - P1, P3 - P1));
  const double rt = r + 2.220446049250313e-16;  // radius + epsilon<double>
  double dist = dot(c - P1, n);
  if (dist < 0) {
    dist = -dist;
    n = dneg(n);
  }
  if (!(dist < rt)) return false;
  bool has = false;
  d3 cp{0, 0, 0};
  if (project_in(P1, P2, P3, n, c)) {
    has = true;
    cp = c - n * dist;
  } else {
    const double r2 = rt * rt;
    d3 near;
    if (seg_sqr(P1, P2, c, near) < r2) { has = true; cp = near; }
    if (seg_sqr(P2, P3, c, near) < r2) { has = true; cp = near; }
    if (seg_sqr(P3, P1, c, near) < r2) { has = true; cp = near; }
  }
  if (!has) return false;
  const d3 ctc = cp - c;
  const double d2 = dsq(ctc);
  if (!(d2 < rt * rt)) return false;
  pos = cp;
  if (d2 > 0) {
    normal = dnormalized(ctc);
    depth = -(r - sqrt(d2));
  } else {
    normal = dneg(n);
    depth = -r;
  }
  return true;
}

__device__ __forceinline__ void put(float* o, f3 pos, f3 nrm, float depth, uint32_t status) {
  o[0] = pos.x; o[1] = pos.y; o[2] = pos.z;
  o[3] = nrm.x; o[4] = nrm.y; o[5] = nrm.z;
  o[6] = depth;
  o[7] = __uint_as_float(status);
}

// Contact status bits (the eighth float of a contact): 0-7 EPA status + 1
// (0 = closed form), bit 8 no contact (GJK or EPA found none: the reference
// adds no contact there).
constexpr uint32_t kMcNone = 1u << 8;

__global__ void __launch_bounds__(kMcWarps * 32) mesh_contact_kernel(MeshShapeArgs m) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  EpaSmem<kMcF, kMcV>& P = reinterpret_cast<EpaSmem<kMcF, kMcV>*>(smem_raw)[threadIdx.x >> 5];
  const unsigned lane = threadIdx.x & 31u;
  const uint64_t total = (uint64_t)m.n * m.max_contacts;
  const uint64_t nw = (uint64_t)gridDim.x * kMcWarps;
  // contacts differ in EPA work: with m.contact_next a warp takes its next
  // kMcTake slots as it finishes (empty slots cost a count check each)
  constexpr uint32_t kMcTake = 4;
  auto take = [&](uint64_t done) -> uint64_t {
    if (!m.contact_next) return done + nw;
    if ((done + 1) % kMcTake != 0) return done + 1;
    uint32_t k = 0;
    if (lane == 0) k = atomicAdd(m.contact_next, kMcTake);
    return (uint64_t)__shfl_sync(0xFFFFFFFFu, k, 0);
  };
  const uint64_t first = m.contact_next ? take(kMcTake - 1) : (uint64_t)blockIdx.x * kMcWarps + (threadIdx.x >> 5);
  for (uint64_t item = first; item < total; item = take(item)) {
    const uint32_t q = (uint32_t)(item / m.max_contacts), slot = (uint32_t)(item % m.max_contacts);
    if (slot >= __ldg(m.counts + q)) continue;  // warp-uniform
    float* out = m.contacts + 8 * item;
    const uint32_t sid = __ldg(m.shape_ids + q);
    const int32_t tri = __ldg(m.tri_ids + item);
    if (sid >= m.n_shapes || tri < 0 || (uint32_t)tri >= m.mesh.n_tris) {
      if (lane == 0) put(out, mk3(0, 0, 0), mk3(0, 0, 1), 0.f, kMcNone);
      continue;
    }
    Pose X;  // the shape in the mesh frame
    {
      const float4 q0 = __ldg(m.poses + 3 * (size_t)q), q1 = __ldg(m.poses + 3 * (size_t)q + 1),
                   q2 = __ldg(m.poses + 3 * (size_t)q + 2);
      X.r[0] = q0.x; X.r[1] = q0.y; X.r[2] = q0.z; X.r[3] = q0.w;
      X.r[4] = q1.x; X.r[5] = q1.y; X.r[6] = q1.z; X.r[7] = q1.w;
      X.r[8] = q2.x;
      X.t = mk3(q2.y, q2.z, q2.w);
    }
    const ShapeDev shp = load_shape(m.shapes, sid);
    if (shp.type == kSphere) {
      if (lane == 0) {
        const f3 P1 = ldv(m.mesh.tris, (uint32_t)tri, 0), P2 = ldv(m.mesh.tris, (uint32_t)tri, 1),
                 P3 = ldv(m.mesh.tris, (uint32_t)tri, 2);
        d3 pos, nrm;
        double depth;
        if (sphere_tri_contact((double)shp.p0, tod(X.t), tod(P1), tod(P2), tod(P3), pos, nrm, depth))
          put(out, mk3((float)pos.x, (float)pos.y, (float)pos.z), mk3((float)-nrm.x, (float)-nrm.y, (float)-nrm.z),
              (float)depth, 0u);
        else
          put(out, mk3(0, 0, 0), mk3(0, 0, 1), 0.f, kMcNone);
      }
      __syncwarp();
      continue;
    }
    // the triangle in the shape's frame: X^-1
    Pose Xi;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) Xi.r[3 * r + c] = X.r[3 * c + r];
    Xi.t = -Xi.rot(X.t);
    // GJK on lane 0 (GJKSolver's guess (1, 0, 0), searched from its negative)
    int rank = 0, gst = 0;
    f3 spa[4], spb[4];
    if (lane == 0) {
      MinkowskiSupport<1> s1;
      s1.A = shp;
      s1.B.type = kTriangle;
      s1.B.vofs = 3 * (uint32_t)tri;
      s1.B.nv = 3;
      s1.B.p0 = s1.B.p1 = s1.B.p2 = 0.f;
      s1.pose = Xi;
      s1.verts = m.verts;
      s1.hull = m.mesh.tris;
      s1.g = Group<1>::make();
      Simplex s0;
      gst = gjk_evaluate(s1, mk3(-1.f, 0.f, 0.f), m.gjk_tol, m.gjk_max_iter, false, s0).status;
      rank = s0.rank;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        spa[i] = s0.a[i];
        spb[i] = s0.b[i];
      }
    }
    gst = __shfl_sync(0xFFFFFFFFu, gst, 0);
    rank = __shfl_sync(0xFFFFFFFFu, rank, 0);
    if (gst != kGjkIntersect) {
      if (lane == 0) put(out, mk3(0, 0, 0), mk3(0, 0, 1), 0.f, kMcNone);
      __syncwarp();
      continue;
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      spa[i] = mk3(__shfl_sync(0xFFFFFFFFu, spa[i].x, 0), __shfl_sync(0xFFFFFFFFu, spa[i].y, 0),
                   __shfl_sync(0xFFFFFFFFu, spa[i].z, 0));
      spb[i] = mk3(__shfl_sync(0xFFFFFFFFu, spb[i].x, 0), __shfl_sync(0xFFFFFFFFu, spb[i].y, 0),
                   __shfl_sync(0xFFFFFFFFu, spb[i].z, 0));
    }
    TriSupport32 sup;
    sup.A = shp;
    sup.pose = Xi;
    sup.verts = m.verts;
    sup.t0 = ldv(m.mesh.tris, (uint32_t)tri, 0);
    sup.t1 = ldv(m.mesh.tris, (uint32_t)tri, 1);
    sup.t2 = ldv(m.mesh.tris, (uint32_t)tri, 2);
    sup.g = Group<32>::make();
    EpaWarp<kMcF, kMcV, TriSupport32> E{P, sup, m.epa_tol, lane, 0, 0, 0, 0, 0u};
    const EpaResult er = E.run(rank < 1 ? 1 : (rank > 4 ? 4 : rank), spa, spb, m.epa_max_iter, kMcF, true);
    if (lane == 0) {
      if (er.status == kEpaFailed) {
        put(out, mk3(0, 0, 0), mk3(0, 0, 1), 0.f, kMcNone | (uint32_t)(er.status + 1));
      } else {
        // pos: the midpoint of the witness points; normal: p0 - p1 (unit, z when zero), in the mesh
        // frame, reversed; depth: EPA's
        const f3 mid = (er.p0 + er.p1) * 0.5f;
        f3 nv = er.p0 - er.p1;
        nv = sqn(nv) > 0.f ? normalized(nv) : mk3(0.f, 0.f, 1.f);
        put(out, X.apply(mid), -X.rot(nv), er.depth, (uint32_t)(er.status + 1));
      }
    }
    __syncwarp();
  }
}

size_t mc_smem_bytes() { return (size_t)kMcWarps * sizeof(EpaSmem<kMcF, kMcV>); }

}  // namespace

cudaError_t launch_mesh_contacts(const MeshShapeArgs& m, int num_sms, cudaStream_t st) {
  if (m.n == 0 || !m.contacts) return cudaSuccess;
  // per launch: the attribute belongs to the current device, and contexts may sit on different devices
  const cudaError_t e = cudaFuncSetAttribute(mesh_contact_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)mc_smem_bytes());
  if (e != cudaSuccess) return e;
  // three 4-warp CTAs of 74 KB fit an SM's shared memory
  mesh_contact_kernel<<<num_sms * 3, kMcWarps * 32, mc_smem_bytes(), st>>>(m);
  return cudaGetLastError();
}

}  // namespace fclg
