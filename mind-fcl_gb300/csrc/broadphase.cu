// Broadphase over a set of posed objects (shape of the context, world pose):
// every pair whose world AABBs overlap, and the narrowphase pair records of
// a candidate list.
//
// The AABBs are CollisionObject::computeAABB's (narrowphase/collision_object-
// inl.h:141-154): the shape's local AABB (computeBV<AABB> at the identity,
// geometry/shape/utility-inl.h) translated when the rotation is exactly the
// identity, otherwise the cube of half size |local half diagonal| about the
// transformed local centre.  The pair set is BinaryAABB_Tree::SelfCollision's
// (broadphase/binary_AABB_tree-inl.h): AABB::overlap, touching boxes included.
// The reference walks a binary AABB tree; here the boxes are sorted by their
// lower x bound (a stable LSD radix sort, 8-bit digits) and swept: box k of the
// sorted order tests the boxes after it while their lower x bound does not
// exceed its upper one.  Pairs go to a capped list through an atomic counter;
// the count is exact even when the list overflows.
#include "broadphase.h"
#include "device_math.cuh"

namespace fclg {

namespace {

constexpr int kSortTile = 1024;  // keys per block and pass (one warp walks them in order)

// IEEE float -> unsigned key with the same order (negative floats reversed).
__device__ __forceinline__ uint32_t float_key(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// Local AABB of every shape (computeBV<AABB>(shape, identity)): box
// +-side / 2; sphere +-r; capsule (r, r, lz / 2 + r); cylinder (r, r, lz / 2);
// hull the extent of its vertices.  lo / hi: float4 per shape.
__global__ void local_aabb_kernel(const int4* __restrict__ shapes, const float4* __restrict__ verts, uint32_t n,
                                  float4* __restrict__ lo, float4* __restrict__ hi) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const ShapeDev s = load_shape(shapes, i);
    f3 a, b;
    switch (s.type) {
      case kBox: b = mk3(s.p0, s.p1, s.p2); a = -b; break;
      case kSphere: b = mk3(s.p0, s.p0, s.p0); a = -b; break;
      case kCapsule: b = mk3(s.p0, s.p0, s.p1 + s.p0); a = -b; break;
      case kCylinder: b = mk3(s.p0, s.p0, s.p1); a = -b; break;
      case kConvex: {
        a = mk3(INFINITY, INFINITY, INFINITY);
        b = -a;
        for (uint32_t k = 0; k < s.nv; ++k) {
          const float4 q = __ldg(verts + s.vofs + k);
          a = mk3(fminf(a.x, q.x), fminf(a.y, q.y), fminf(a.z, q.z));
          b = mk3(fmaxf(b.x, q.x), fmaxf(b.y, q.y), fmaxf(b.z, q.z));
        }
        break;
      }
      default: a = b = mk3(0.f, 0.f, 0.f);
    }
    lo[i] = make_float4(a.x, a.y, a.z, 0.f);
    hi[i] = make_float4(b.x, b.y, b.z, 0.f);
  }
}

// World AABB of object i (CollisionObject::computeAABB) and its sort key.
__global__ void object_aabb_kernel(const uint32_t* __restrict__ ids, const float4* __restrict__ poses, uint32_t n,
                                   uint32_t n_shapes, const float4* __restrict__ llo, const float4* __restrict__ lhi,
                                   float4* __restrict__ lo, float4* __restrict__ hi, uint32_t* __restrict__ key,
                                   uint32_t* __restrict__ val) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t s = __ldg(ids + i);
    const float4 q0 = __ldg(poses + 3 * (size_t)i), q1 = __ldg(poses + 3 * (size_t)i + 1),
                 q2 = __ldg(poses + 3 * (size_t)i + 2);
    const float r[9] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w, q2.x};
    const f3 t = mk3(q2.y, q2.z, q2.w);
    f3 a, b;
    if (s >= n_shapes) {
      // no shape: an empty box far away that overlaps nothing
      a = mk3(INFINITY, INFINITY, INFINITY);
      b = -a;
    } else {
      const float4 l = __ldg(llo + s), h = __ldg(lhi + s);
      const bool identity = r[0] == 1.f && r[4] == 1.f && r[8] == 1.f && r[1] == 0.f && r[2] == 0.f &&
                            r[3] == 0.f && r[5] == 0.f && r[6] == 0.f && r[7] == 0.f;
      if (identity) {
        a = mk3(l.x, l.y, l.z) + t;
        b = mk3(h.x, h.y, h.z) + t;
      } else {
        const f3 c = (mk3(l.x, l.y, l.z) + mk3(h.x, h.y, h.z)) * 0.5f;
        const float rad = nrm(mk3(l.x, l.y, l.z) - c);
        const f3 cw = mk3(fmaf(r[2], c.z, fmaf(r[1], c.y, r[0] * c.x)), fmaf(r[5], c.z, fmaf(r[4], c.y, r[3] * c.x)),
                          fmaf(r[8], c.z, fmaf(r[7], c.y, r[6] * c.x))) + t;
        a = cw - mk3(rad, rad, rad);
        b = cw + mk3(rad, rad, rad);
      }
    }
    lo[i] = make_float4(a.x, a.y, a.z, 0.f);
    hi[i] = make_float4(b.x, b.y, b.z, 0.f);
    key[i] = float_key(a.x);
    val[i] = i;
  }
}

// Radix pass, step 1: digit counts of each tile, stored digit-major.
__global__ void radix_hist_kernel(const uint32_t* __restrict__ key, uint32_t n, int shift, uint32_t* __restrict__ hist,
                                  uint32_t n_tiles) {
  __shared__ uint32_t c[256];
  for (int d = threadIdx.x; d < 256; d += blockDim.x) c[d] = 0;
  __syncthreads();
  const uint32_t tile = blockIdx.x;
  const uint32_t b = tile * kSortTile, e = min(n, b + kSortTile);
  for (uint32_t i = b + threadIdx.x; i < e; i += blockDim.x) atomicAdd(&c[(__ldg(key + i) >> shift) & 0xFFu], 1u);
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += blockDim.x) hist[(size_t)d * n_tiles + tile] = c[d];
}

// Step 2: exclusive scan of the digit-major counts (one block).
__global__ void radix_scan_kernel(uint32_t* __restrict__ hist, uint32_t m) {
  __shared__ uint32_t part[1024];
  const uint32_t per = (m + blockDim.x - 1) / blockDim.x;
  const uint32_t b = threadIdx.x * per, e = min(m, b + per);
  uint32_t s = 0;
  for (uint32_t i = b; i < e; ++i) s += hist[i];
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t acc = 0;
    for (uint32_t k = 0; k < blockDim.x; ++k) {
      const uint32_t v = part[k];
      part[k] = acc;
      acc += v;
    }
  }
  __syncthreads();
  uint32_t acc = part[threadIdx.x];
  for (uint32_t i = b; i < e; ++i) {
    const uint32_t v = hist[i];
    hist[i] = acc;
    acc += v;
  }
}

// Step 3: stable scatter.  One warp per tile walks it 32 keys at a time, in
// order; keys with the same digit in one round are ranked by lane.
__global__ void radix_scatter_kernel(const uint32_t* __restrict__ key, const uint32_t* __restrict__ val, uint32_t n,
                                     int shift, const uint32_t* __restrict__ hist, uint32_t n_tiles,
                                     uint32_t* __restrict__ key_out, uint32_t* __restrict__ val_out) {
  __shared__ uint32_t off[256];
  const uint32_t tile = blockIdx.x;
  const unsigned lane = threadIdx.x;
  for (int d = lane; d < 256; d += 32) off[d] = hist[(size_t)d * n_tiles + tile];
  __syncwarp();
  const uint32_t b = tile * kSortTile, e = min(n, b + kSortTile);
  for (uint32_t base = b; base < e; base += 32) {
    const uint32_t i = base + lane;
    const bool ok = i < e;
    const uint32_t k = ok ? key[i] : 0u;
    const uint32_t d = ok ? ((k >> shift) & 0xFFu) : 256u;
    const unsigned peers = __match_any_sync(0xFFFFFFFFu, d);
    const unsigned lower = peers & ((1u << lane) - 1u);
    const uint32_t start = ok ? off[d] : 0u;
    __syncwarp();
    if (ok) {
      const uint32_t dst = start + (uint32_t)__popc(lower);
      key_out[dst] = k;
      val_out[dst] = val[i];
      if (lower == 0) off[d] = start + (uint32_t)__popc(peers);  // the group's first lane advances the digit
    }
    __syncwarp();
  }
}

// The sweep: sorted box k against the boxes after it while they can overlap in x.
__global__ void sweep_kernel(const uint32_t* __restrict__ order, const float4* __restrict__ lo,
                             const float4* __restrict__ hi, uint32_t n, uint32_t split, uint32_t* __restrict__ pairs,
                             uint32_t cap, uint32_t* __restrict__ count) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const uint32_t i = order[k];
    const float4 la = __ldg(lo + i), ha = __ldg(hi + i);
    for (uint32_t m = k + 1; m < n; ++m) {
      const uint32_t j = order[m];
      const float4 lb = __ldg(lo + j);
      if (lb.x > ha.x) break;  // sorted by lower x: no later box reaches back
      const float4 hb = __ldg(hi + j);
      // AABB::overlap (math/bv/AABB-inl.h): apart only if one box starts past the other's end
      if (la.y > hb.y || lb.y > ha.y || la.z > hb.z || lb.z > ha.z || la.x > hb.x) continue;
      if (split && ((i < split) == (j < split))) continue;  // two sets: only pairs across them
      const uint32_t slot = atomicAdd(count, 1u);
      if (slot < cap) {
        const uint32_t lo_i = min(i, j), hi_i = max(i, j);
        pairs[2 * (size_t)slot] = lo_i;
        pairs[2 * (size_t)slot + 1] = split ? hi_i - split : hi_i;
      }
    }
  }
}

// Narrowphase record of candidate (i, j): shape_ids[i] at the origin, shape_ids[j]
// posed by X_i^-1 X_j (the relative transform fcl's narrowphase works in).
__global__ void pairs_kernel(const uint32_t* __restrict__ ids, const float4* __restrict__ poses,
                             const uint32_t* __restrict__ cand, uint32_t m, float4* __restrict__ out) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
    const uint32_t i = __ldg(cand + 2 * (size_t)k), j = __ldg(cand + 2 * (size_t)k + 1);
    float a[12], b[12];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const float4 u = __ldg(poses + 3 * (size_t)i + q), v = __ldg(poses + 3 * (size_t)j + q);
      a[4 * q] = u.x; a[4 * q + 1] = u.y; a[4 * q + 2] = u.z; a[4 * q + 3] = u.w;
      b[4 * q] = v.x; b[4 * q + 1] = v.y; b[4 * q + 2] = v.z; b[4 * q + 3] = v.w;
    }
    // R = Ra^T Rb, t = Ra^T (tb - ta)
    float R[9], t[3];
    const float dt[3] = {b[9] - a[9], b[10] - a[10], b[11] - a[11]};
#pragma unroll
    for (int r = 0; r < 3; ++r) {
#pragma unroll
      for (int c = 0; c < 3; ++c) R[3 * r + c] = fmaf(a[6 + r], b[6 + c], fmaf(a[3 + r], b[3 + c], a[r] * b[c]));
      t[r] = fmaf(a[6 + r], dt[2], fmaf(a[3 + r], dt[1], a[r] * dt[0]));
    }
    float4* o = out + 4 * (size_t)k;
    o[0] = make_float4(__uint_as_float(__ldg(ids + i)), __uint_as_float(__ldg(ids + j)), R[0], R[1]);
    o[1] = make_float4(R[2], R[3], R[4], R[5]);
    o[2] = make_float4(R[6], R[7], R[8], t[0]);
    o[3] = make_float4(t[1], t[2], 0.f, 0.f);
  }
}

}  // namespace

size_t broadphase_scratch_bytes(uint32_t n_objects, uint32_t n_shapes) {
  const size_t tiles = (n_objects + kSortTile - 1) / kSortTile;
  auto r = [](size_t b) { return (b + 255) & ~(size_t)255; };
  return 2 * r((size_t)n_shapes * 16) + 2 * r((size_t)n_objects * 16) + 4 * r((size_t)n_objects * 4) +
         r(256 * tiles * 4);
}

cudaError_t launch_broadphase(const BroadphaseArgs& a, void* scratch, cudaStream_t st) {
  const uint32_t n = a.n;
  if (cudaMemsetAsync(a.count, 0, sizeof(uint32_t), st) != cudaSuccess) return cudaGetLastError();
  if (n == 0) return cudaSuccess;
  const uint32_t tiles = (n + kSortTile - 1) / kSortTile;
  char* p = static_cast<char*>(scratch);
  auto take = [&](size_t bytes) {
    char* q = p;
    p += (bytes + 255) & ~(size_t)255;
    return q;
  };
  float4* llo = reinterpret_cast<float4*>(take((size_t)a.n_shapes * 16));
  float4* lhi = reinterpret_cast<float4*>(take((size_t)a.n_shapes * 16));
  float4* lo = a.aabb_lo ? a.aabb_lo : reinterpret_cast<float4*>(take((size_t)n * 16));
  float4* hi = a.aabb_hi ? a.aabb_hi : reinterpret_cast<float4*>(take((size_t)n * 16));
  uint32_t* k0 = reinterpret_cast<uint32_t*>(take((size_t)n * 4));
  uint32_t* v0 = reinterpret_cast<uint32_t*>(take((size_t)n * 4));
  uint32_t* k1 = reinterpret_cast<uint32_t*>(take((size_t)n * 4));
  uint32_t* v1 = reinterpret_cast<uint32_t*>(take((size_t)n * 4));
  uint32_t* hist = reinterpret_cast<uint32_t*>(take(256 * (size_t)tiles * 4));
  const int tb = 256;
  local_aabb_kernel<<<(a.n_shapes + tb - 1) / tb, tb, 0, st>>>(a.shapes, a.verts, a.n_shapes, llo, lhi);
  object_aabb_kernel<<<(n + tb - 1) / tb, tb, 0, st>>>(a.shape_ids, a.poses, n, a.n_shapes, llo, lhi, lo, hi, k0, v0);
  for (int shift = 0; shift < 32; shift += 8) {
    radix_hist_kernel<<<tiles, 256, 0, st>>>(k0, n, shift, hist, tiles);
    radix_scan_kernel<<<1, 1024, 0, st>>>(hist, 256 * tiles);
    radix_scatter_kernel<<<tiles, 32, 0, st>>>(k0, v0, n, shift, hist, tiles, k1, v1);
    uint32_t* t = k0; k0 = k1; k1 = t;
    t = v0; v0 = v1; v1 = t;
  }
  sweep_kernel<<<(n + tb - 1) / tb, tb, 0, st>>>(v0, lo, hi, n, a.split, a.pairs, a.cap, a.count);
  return cudaGetLastError();
}

int broadphase_launches() { return 2 + 4 * 3 + 1; }

cudaError_t launch_object_pairs(const uint32_t* shape_ids, const float* poses, const uint32_t* cand, uint32_t m,
                                void* out_pairs, cudaStream_t st) {
  if (m == 0) return cudaSuccess;
  const int tb = 256;
  pairs_kernel<<<(m + tb - 1) / tb, tb, 0, st>>>(shape_ids, reinterpret_cast<const float4*>(poses), cand, m,
                                                 static_cast<float4*>(out_pairs));
  return cudaGetLastError();
}

}  // namespace fclg
