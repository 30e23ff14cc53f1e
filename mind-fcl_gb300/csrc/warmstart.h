// Learned warm start for GJK: the direction model's interface to the query
// path (api.cu).  The model and its kernels live in warmstart.cu.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

struct fclg_warmstart;

namespace fclg {

// Writes the model's unit search direction for each pair (float[n][3]) on
// stream st.  Returns the CUDA error of the launch.
cudaError_t warmstart_predict(fclg_warmstart* ws, const float4* pairs, uint32_t n, float* guess, cudaStream_t st);
int warmstart_device(const fclg_warmstart* ws);

}  // namespace fclg
