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
  const double* size;   // [n_nodes] FP64 |extent|^2 of the reference's box (the descend key)
};

struct MeshArgs {
  MeshDev a, b;
  const float4* poses;  // 3 float4 per pose: rotation row-major, translation (b in a's frame)
  uint32_t n_poses;
  uint32_t max_contacts;  // >= 1
  uint8_t* flags;         // [n_poses]
  uint32_t* counts;       // [n_poses]
  int32_t* pairs;         // [n_poses][max_contacts][2] triangle ids (a, b)
  uint32_t* status;       // [n_poses] or null: bit 0 stack overflow, bit 1 round limit, bit 2 path too long
  // per-warp contact buffers for max_contacts above the shared-memory buffer
  // (mesh_contact_buffer_len entries per warp, mesh_collide_warps warps)
  unsigned long long* cbuf_key = nullptr;
  int2* cbuf_pair = nullptr;
  uint32_t cbuf_len = 0;
  // optional traffic counters (profiling): [0] node pairs whose boxes were
  // tested, [1] triangle pairs tested
  unsigned long long* counters = nullptr;
  // optional, zero before the launch: poses taken so far; each warp takes its
  // next pose there as it finishes one (a persistent grid), else warp w takes
  // poses w, w + W, ...
  uint32_t* next = nullptr;
};

cudaError_t launch_mesh_collide(const MeshArgs& m, int blocks, cudaStream_t st);
// Global contact-buffer entries per warp a request with max_contacts needs (0:
// it fits in shared memory), and the warps a launch of `blocks` CTAs runs.
int mesh_contact_buffer_len(uint32_t max_contacts);
int mesh_collide_warps(int blocks);
// CTAs of the mesh-mesh kernel that fit on the device at once.
int mesh_collide_resident_blocks(int num_sms);

// Mesh against shapes of the context (mesh_shape.cu): query i = shape
// shape_ids[i] posed by poses[i] in the mesh frame.
struct MeshShapeArgs {
  MeshDev mesh;
  const int4* shapes;     // fclg_shape[n_shapes]
  const float4* verts;    // hull vertices, xyzw
  uint32_t n_shapes;
  const uint32_t* shape_ids;  // [n]
  const float4* poses;        // 3 float4 per query: rotation row-major, translation
  uint32_t n;
  uint32_t max_contacts;      // >= 1
  float gjk_tol;              // MPR / GJK leaves (GJKSolver defaults 1e-6, 128)
  int gjk_max_iter;
  uint8_t* flags;             // [n]
  uint32_t* counts;           // [n]
  int32_t* tri_ids;           // [n][max_contacts]
  uint32_t* status;           // [n] or null: bit 0 stack overflow, bit 1 round limit, bit 2 bad shape id
  // penetration on: leaves other than spheres decide by GJK (the test that
  // feeds EPA), and contacts[n][max_contacts][8] receive pos (3), normal (3),
  // depth and the EPA status bits of each reported triangle
  float* contacts = nullptr;
  float epa_tol = 1e-6f;      // GJKSolver defaults: 256 faces, 255 iterations, 1e-6
  int epa_max_iter = 255;
  // per-warp contact buffers for max_contacts above the shared-memory buffer
  // (mesh_contact_buffer_len entries per warp, mesh_shape_warps warps)
  unsigned long long* cbuf_key = nullptr;
  int2* cbuf_val = nullptr;
  uint32_t cbuf_len = 0;
  // optional, zero before the launch: queries taken so far (as MeshArgs::next)
  uint32_t* next = nullptr;
  // optional, zero before the contact launch: contact slots taken so far by
  // its warps (launch_mesh_contacts)
  uint32_t* contact_next = nullptr;
};

cudaError_t launch_mesh_shape(const MeshShapeArgs& m, int blocks, cudaStream_t st);
int mesh_shape_warps(int blocks);
// CTAs of the mesh-shape kernel that fit on the device at once.
int mesh_shape_resident_blocks(int num_sms, bool penetration);
// The contacts of the triangles a penetration-mode launch reported
// (mesh_contact.cu): sphere leaves in closed form, the others by GJK + EPA.
cudaError_t launch_mesh_contacts(const MeshShapeArgs& m, int num_sms, cudaStream_t st);

}  // namespace fclg
