// Host-side BVH build for triangle meshes (mesh_build.cpp).
#pragma once
#include <cstdint>
#include <vector>

namespace fclg {

// One 64-byte BVH node (same layout as fclg_mesh_node in include/fclg.h).
struct MeshNodeRec {
  float axis[9];    // row-major; columns are the box axes
  float center[3];
  float extent[3];  // half sizes
  int32_t child;    // >= 0: children child, child + 1; < 0: leaf of triangle -(child + 1)
};
static_assert(sizeof(MeshNodeRec) == 64, "node layout");

// Builds the reference's OBBRSS tree (2 * nt - 1 nodes, root 0, children of
// a node in adjacent slots) with FP32 boxes that contain their triangles, and
// the triangle soup (3 x xyzw per triangle, in input order).  sizes (if not
// null) receives each node's FP64 |extent|^2 as the reference computes it,
// depth (if not null) the deepest node's level (root 0).  Returns 0, or -1
// for an empty mesh, -2 for a vertex index out of range.
int build_obb_bvh(const float* vertices_xyz, uint32_t nv, const int32_t* tris, uint32_t nt,
                  std::vector<MeshNodeRec>& nodes, std::vector<float>& tri_xyzw, std::vector<double>* sizes = nullptr,
                  uint32_t* depth = nullptr);

}  // namespace fclg
