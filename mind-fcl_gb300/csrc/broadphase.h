// Launch interface of the broadphase (broadphase.cu).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace fclg {

struct BroadphaseArgs {
  const int4* shapes;       // the context's fclg_shape table
  const float4* verts;      // its hull vertices
  uint32_t n_shapes;
  const uint32_t* shape_ids;  // [n] shape of each object
  const float4* poses;        // [n] 3 float4: world rotation row-major, translation
  uint32_t n;
  uint32_t* pairs;            // [cap][2] overlapping object pairs (i < j)
  uint32_t cap;
  uint32_t* count;            // [1] number of overlapping pairs (may exceed cap)
  float4* aabb_lo;            // optional [n]: the world AABBs
  float4* aabb_hi;
  uint32_t split;             // 0: every pair; else objects [0, split) and [split, n) are two sets and only
                              // pairs across them count, written as (index in the first, index in the second)
};

// Device scratch the launch needs (byte size; any 256-byte aligned buffer).
size_t broadphase_scratch_bytes(uint32_t n_objects, uint32_t n_shapes);
cudaError_t launch_broadphase(const BroadphaseArgs& a, void* scratch, cudaStream_t st);
// Kernels one broadphase launches.
int broadphase_launches();
// Narrowphase records (fclg_pair) of candidate object pairs.
cudaError_t launch_object_pairs(const uint32_t* shape_ids, const float* poses, const uint32_t* cand, uint32_t m,
                                void* out_pairs, cudaStream_t st);

}  // namespace fclg
