// Internal launch interface between the C ABI (api.cu) and the kernels.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "device_math.cuh"

namespace fclg {

struct BatchArgs {
  const int4* shapes;     // fclg_shape[n_shapes]
  const float4* verts;    // xyzw
  const float4* pairs;    // fclg_pair[n_pairs]
  const float* guess;     // optional float[n_pairs][3]: GJKSolver::gjk_guess per pair
  float4* results;        // fclg_result[n_pairs]
  uint32_t n_pairs;
  uint32_t n_shapes;
};

// Scratch of a query batch: the overlapping pairs handed from the GJK pass to
// the EPA pass.  count must be zero before the GJK pass.
struct EpaQueue {
  uint32_t* count;        // [1]
  uint32_t* list;         // [capacity] pair indices
  float4* rec;            // [capacity][7] final GJK simplex (rank, support points)
};
constexpr size_t kEpaRecordBytes = 7 * sizeof(float4);

cudaError_t launch_gjk(const BatchArgs& b, const QueryParams& prm, const EpaQueue& q, int lanes, cudaStream_t st);
cudaError_t prepare_epa();
cudaError_t launch_epa(const BatchArgs& b, const QueryParams& prm, const EpaQueue& q, int blocks, cudaStream_t st);
size_t epa_smem_bytes();
int epa_max_faces_supported();

}  // namespace fclg
