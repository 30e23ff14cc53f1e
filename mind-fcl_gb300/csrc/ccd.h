// Launch interface of the translational continuous-collision pass (ccd_pass.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "kernels.h"

namespace fclg {

// TimeOfCollisionRequestType (narrowphase/detail/ccd/ccd_request.h:11-17).
constexpr int kTocNone = 0, kTocBox = 1, kTocSample = 2;

// Result status bits: 0-1 the swept MPR's status (0 Intersect, 1 Separated,
// 2 Failed, 3 not run), 2 the box interval test ran, 3 it found the boxes
// disjoint, 4 a shape id out of range.
constexpr uint32_t kCcdNoMpr = 3u, kCcdBoxTested = 4u, kCcdBoxDisjoint = 8u, kCcdBadShape = 16u;

struct CcdParams {
  int toc_type;
  int max_iter;     // MPR (ContinuousCollisionRequest::max_gjk_iterations, 128)
  float tol;        // MPR (gjk_tolerance, 1e-6)
  double zero_tol;  // zero_movement_tolerance (1e-4)
};

// Local AABB of every hull into aabb (2 float4 per shape: lo, hi).
cudaError_t launch_hull_aabbs(const int4* shapes, const float4* verts, uint32_t n_shapes, float4* aabb,
                              cudaStream_t st);
// One pass over b's pairs: disp[i] = (unit axis in a's frame, distance),
// aabb = the hull boxes (read by the approximate request), order = the pairs
// in shape-class order (or null: index order), out[i] = fclg_ccd_result;
// next (optional, zero before the launch): the counter the persistent grid's
// warps take their pairs from.
cudaError_t launch_ccd(const BatchArgs& b, const float4* disp, const float4* aabb, const CcdParams& prm,
                       const uint32_t* order, float4* out, int num_sms, cudaStream_t st, uint32_t* next = nullptr);

}  // namespace fclg
