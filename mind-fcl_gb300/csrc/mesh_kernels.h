// Launch interface of the mesh-mesh kernel (mesh_query.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace fclg {

struct MeshDev {
  const float4* nodes;  // 4 float4 per node (fclg_mesh_node)
  const float4* tris;   // 3 float4 per triangle (x, y, z, 0)
  uint32_t n_nodes;
  uint32_t n_tris;
};

struct MeshArgs {
  MeshDev a, b;
  const float4* poses;  // 3 float4 per pose: rotation row-major, translation (b in a's frame)
  uint32_t n_poses;
  uint32_t max_contacts;  // >= 1
  uint8_t* flags;         // [n_poses]
  uint32_t* counts;       // [n_poses]
  int32_t* pairs;         // [n_poses][max_contacts][2] triangle ids (a, b)
  uint32_t* status;       // [n_poses] or null: bit 0 stack overflow, bit 1 round limit
};

cudaError_t launch_mesh_collide(const MeshArgs& m, int blocks, cudaStream_t st);

}  // namespace fclg
