// Bucketing of a pair batch by shape class (a device-side counting sort).
//
// The reference dispatches each pair through a NODE_TYPE x NODE_TYPE function
// table (narrowphase/detail/collision_func_matrix-inl.h:585-858); on the GPU the
// same role is played by sorting the batch so that every warp runs one support
// routine pair: warps over mixed types would execute every support routine of
// the mix in turn.  Shape classes: box, sphere, capsule, cylinder, convex hulls
// up to `big_nv` vertices in five bins of vertex count (a lane's hull scan
// takes as long as its vertex count, and a warp as long as its largest hull,
// so the warps of a bin scan hulls within a factor of two of each other), and
// hulls above `big_nv`; pairs with such a hull sort last so a second launch can
// give them more lanes per pair.
//
//   classify  per pair: class key + block histogram, merged with one atomic
//             per (block, key)
//   scan      one block: exclusive scan of the histogram, bucket cursors and
//             the [begin, end) ranges of the two launches
//   scatter   per pair: rank within the block's share of its bucket, block
//             share reserved with one atomic per (block, key)
#include "kernels.h"

namespace fclg {

namespace {

constexpr uint32_t kBigHull = 4 + kHullBins;

__device__ __forceinline__ uint32_t shape_class(int4 h, uint32_t big_nv) {
  switch (h.x) {
    case kBox: return 0;
    case kSphere: return 1;
    case kCapsule: return 2;
    case kCylinder: return 3;
    default: {
      const uint32_t nv = (uint32_t)h.z;
      if (nv > big_nv) return kBigHull;
      const int lg = 31 - __clz((int)(nv | 1u));  // floor(log2(nv))
      return 4u + (uint32_t)min(max(lg - 3, 0), kHullBins - 1);
    }
  }
}

}  // namespace

__global__ void __launch_bounds__(256) classify_pairs(const float4* __restrict__ pairs, const int4* __restrict__ shapes,
                                                      uint32_t n, uint32_t n_shapes, uint32_t big_nv,
                                                      uint8_t* __restrict__ keys, uint32_t* __restrict__ hist) {
  __shared__ uint32_t sh[kBucketKeys];
  for (int k = threadIdx.x; k < kBucketKeys; k += blockDim.x) sh[k] = 0;
  __syncthreads();
  const uint32_t pid = blockIdx.x * blockDim.x + threadIdx.x;
  if (pid < n) {
    const float4 q = __ldg(pairs + 4 * (size_t)pid);
    const uint32_t a = __float_as_uint(q.x), b = __float_as_uint(q.y);
    uint32_t key = 0;
    if (a < n_shapes && b < n_shapes) {
      const uint32_t ca = shape_class(__ldg(shapes + 2 * (size_t)a), big_nv);
      const uint32_t cb = shape_class(__ldg(shapes + 2 * (size_t)b), big_nv);
      const bool big = ca == kBigHull || cb == kBigHull;
      key = (big ? kBucketSmallKeys : 0u) + ca * kShapeClasses + cb;
    }
    keys[pid] = (uint8_t)key;
    atomicAdd(&sh[key], 1u);
  }
  __syncthreads();
  for (int k = threadIdx.x; k < kBucketKeys; k += blockDim.x)
    if (sh[k]) atomicAdd(&hist[k], sh[k]);
}

__global__ void scan_buckets(uint32_t* __restrict__ hist, uint32_t* __restrict__ cursor, uint32_t* __restrict__ ranges) {
  // kBucketKeys <= blockDim.x: one thread per key, a Hillis-Steele scan in shared memory
  __shared__ uint32_t s[kBucketKeys];
  const int k = threadIdx.x;
  const uint32_t v = k < kBucketKeys ? hist[k] : 0u;
  if (k < kBucketKeys) s[k] = v;
  __syncthreads();
  for (int off = 1; off < kBucketKeys; off <<= 1) {
    uint32_t t = 0;
    if (k < kBucketKeys && k >= off) t = s[k - off];
    __syncthreads();
    if (k < kBucketKeys) s[k] += t;
    __syncthreads();
  }
  if (k < kBucketKeys) {
    const uint32_t excl = s[k] - v;
    cursor[k] = excl;
    if (k == kBucketSmallKeys) {
      ranges[1] = excl;  // small-pair launch: [0, excl)
      ranges[2] = excl;  // large-pair launch: [excl, n)
    }
    if (k == kBucketKeys - 1) ranges[3] = s[k];
    if (k == 0) ranges[0] = 0;
    hist[k] = 0;  // ready for the next batch
  }
}

__global__ void __launch_bounds__(256) scatter_pairs(const uint8_t* __restrict__ keys, uint32_t n,
                                                     uint32_t* __restrict__ cursor, uint32_t* __restrict__ order) {
  __shared__ uint32_t cnt[kBucketKeys];
  __shared__ uint32_t base[kBucketKeys];
  for (int k = threadIdx.x; k < kBucketKeys; k += blockDim.x) cnt[k] = 0;
  __syncthreads();
  const uint32_t pid = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t key = 0, local = 0;
  if (pid < n) {
    key = keys[pid];
    local = atomicAdd(&cnt[key], 1u);
  }
  __syncthreads();
  for (int k = threadIdx.x; k < kBucketKeys; k += blockDim.x)
    if (cnt[k]) base[k] = atomicAdd(&cursor[k], cnt[k]);
  __syncthreads();
  if (pid < n) order[base[key] + local] = pid;
}

cudaError_t launch_bucketing(const BatchArgs& b, const BucketScratch& s, uint32_t big_nv, cudaStream_t st) {
  if (b.n_pairs == 0) return cudaSuccess;
  const unsigned blocks = (b.n_pairs + 255) / 256;
  classify_pairs<<<blocks, 256, 0, st>>>(b.pairs, b.shapes, b.n_pairs, b.n_shapes, big_nv, s.keys, s.hist);
  scan_buckets<<<1, 256, 0, st>>>(s.hist, s.cursor, s.ranges);
  scatter_pairs<<<blocks, 256, 0, st>>>(s.keys, b.n_pairs, s.cursor, s.order);
  return cudaGetLastError();
}

}  // namespace fclg
