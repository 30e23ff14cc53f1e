// GJK pass launcher: picks the lane count's instantiation (gjk_pass_l*.cu).
#include "gjk_pass.cuh"

namespace fclg {

FCLG_GJK_INSTANTIATE(1)
FCLG_GJK_INSTANTIATE(2)

cudaError_t launch_gjk(const BatchArgs& b, const QueryParams& prm, const EpaQueue& q, int lanes,
                       const uint32_t* order, const uint32_t* range, int blocks, cudaStream_t st) {
  if (b.n_pairs == 0) return cudaSuccess;
  const int threads = 128;
  if (blocks <= 0) {
    const uint64_t total = (uint64_t)b.n_pairs * (uint64_t)lanes;
    blocks = (int)((total + threads - 1) / threads);
  }
  switch (lanes) {
    case 1: return launch_gjk_lanes<1>(b, prm, q, order, range, blocks, st);
    case 2: return launch_gjk_lanes<2>(b, prm, q, order, range, blocks, st);
    case 4: return launch_gjk_lanes<4>(b, prm, q, order, range, blocks, st);
    case 8: return launch_gjk_lanes<8>(b, prm, q, order, range, blocks, st);
    case 16: return launch_gjk_lanes<16>(b, prm, q, order, range, blocks, st);
    case 32: return launch_gjk_lanes<32>(b, prm, q, order, range, blocks, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace fclg
