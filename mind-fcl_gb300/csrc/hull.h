// Convex-hull vertex adjacency for the support walk (hull.cpp).
#pragma once
#include <cstdint>
#include <vector>

namespace fclg {

// Hulls with more vertices than this are walked (the reference's
// kMinVertCountForEdgeWalking, geometry/shape/convex.h:60-61); smaller ones
// are scanned.
constexpr uint32_t kWalkMinVertices = 32;
// Largest vertex degree a packed walk block holds (8 bits of the link word).
constexpr uint32_t kWalkMaxDegree = 255;

// Edge graph of one hull.  Vertices that are not corners of the hull
// (interior, duplicates, or within rounding of a face) have empty rows and are
// never reached from the six starts.
struct HullGraph {
  uint32_t start[6];           // extreme corner along +x, -x, +y, -y, +z, -z
  std::vector<uint32_t> first; // [nv + 1] row starts into adj
  std::vector<uint32_t> adj;   // neighbour vertex indices, each row ascending
};

// False (graph cleared) when the points span no volume or fewer than 4 are given.
bool hull_graph(const float* xyzw, uint32_t nv, HullGraph& g);

// Appends the device walk block of one hull to `out` (4 floats per entry):
//   entries [0, 6)   the six start corners
//   then, per corner, the entries of its neighbours (its row)
// entry = {x, y, z, link}; link (the float's bits) = (row offset in the block
// << 8) | degree, the same word for every entry of one vertex.
// False when a degree exceeds kWalkMaxDegree or the block exceeds 2^24 entries.
bool pack_walk(const float* xyzw, const HullGraph& g, std::vector<float>& out);

}  // namespace fclg
