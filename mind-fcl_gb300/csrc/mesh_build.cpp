// Host-side OBB BVH build for triangle meshes.
//
// Plays the role of the reference's BVHModel<OBBRSS>::beginModel / addSubModel
// / endModel (geometry/bvh/BVH_model-inl.h:136-303, iterativeBuildTree
// :450-570): top-down, one triangle per leaf, children of a node stored next
// to each other, each node's box fitted to its triangles' vertices along the
// principal axes of their covariance (the reference fits OBBRSS the same way,
// geometry/bvh/detail/BV_fitter-inl.h:323-345, math/bv/utility-inl.h), and a
// node split at the mean of its triangle centroids along its longest axis
// (the reference's default mean splitter, BV_splitter-inl.h).  The reference's
// OBBRSS overlap test only reads the OBB (math/bv/OBBRSS-inl.h:132-137), so
// the GPU node is an OBB.
//
// Nodes are stored in FP32 for the kernels; every box is re-measured in FP64
// against its FP32-rounded axes and centre and its extents rounded up, so
// the stored box contains every stored vertex.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "mesh_build.h"

namespace fclg {

namespace {

// Eigen-decomposition of a symmetric 3x3 matrix by cyclic Jacobi rotations.
void jacobi3(const double A_in[9], double evals[3], double evecs[9]) {
  double a[9];
  std::memcpy(a, A_in, sizeof a);
  double v[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  for (int sweep = 0; sweep < 50; ++sweep) {
    const double off = a[1] * a[1] + a[2] * a[2] + a[5] * a[5];
    if (off < 1e-30) break;
    for (int p = 0; p < 2; ++p) {
      for (int q = p + 1; q < 3; ++q) {
        const double apq = a[3 * p + q];
        if (std::abs(apq) < 1e-300) continue;
        const double theta = (a[3 * q + q] - a[3 * p + p]) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::abs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < 3; ++k) {  // A <- J^T A J
          const double akp = a[3 * k + p], akq = a[3 * k + q];
          a[3 * k + p] = c * akp - s * akq;
          a[3 * k + q] = s * akp + c * akq;
        }
        for (int k = 0; k < 3; ++k) {
          const double apk = a[3 * p + k], aqk = a[3 * q + k];
          a[3 * p + k] = c * apk - s * aqk;
          a[3 * q + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < 3; ++k) {
          const double vkp = v[3 * k + p], vkq = v[3 * k + q];
          v[3 * k + p] = c * vkp - s * vkq;
          v[3 * k + q] = s * vkp + c * vkq;
        }
      }
    }
  }
  for (int i = 0; i < 3; ++i) evals[i] = a[4 * i];
  std::memcpy(evecs, v, sizeof v);
}

struct Work {
  int node, begin, end;
};

// Fits node `ni` to triangles perm[b, e); returns the longest box axis index.
int fit_node(const std::vector<double>& V, const std::vector<int32_t>& T, const std::vector<int>& perm, int b, int e,
             MeshNodeRec& out) {
  double mean[3] = {0, 0, 0};
  const int np = 3 * (e - b);
  for (int i = b; i < e; ++i)
    for (int k = 0; k < 3; ++k) {
      const double* p = &V[3 * (size_t)T[3 * (size_t)perm[i] + k]];
      mean[0] += p[0];
      mean[1] += p[1];
      mean[2] += p[2];
    }
  for (double& m : mean) m /= np;
  double C[9] = {0};
  for (int i = b; i < e; ++i)
    for (int k = 0; k < 3; ++k) {
      const double* p = &V[3 * (size_t)T[3 * (size_t)perm[i] + k]];
      const double d[3] = {p[0] - mean[0], p[1] - mean[1], p[2] - mean[2]};
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) C[3 * r + c] += d[r] * d[c];
    }
  double ev[3], U[9];
  jacobi3(C, ev, U);
  int order[3] = {0, 1, 2};
  std::sort(order, order + 3, [&](int x, int y) { return ev[x] > ev[y]; });
  double ax[3][3];
  for (int j = 0; j < 2; ++j)
    for (int r = 0; r < 3; ++r) ax[j][r] = U[3 * r + order[j]];
  // right-handed third axis
  ax[2][0] = ax[0][1] * ax[1][2] - ax[0][2] * ax[1][1];
  ax[2][1] = ax[0][2] * ax[1][0] - ax[0][0] * ax[1][2];
  ax[2][2] = ax[0][0] * ax[1][1] - ax[0][1] * ax[1][0];
  for (auto& a : ax) {
    const double n = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    for (double& x : a) x /= n;
  }
  // FP32 axes (stored: axis matrix row r, column j = ax[j][r])
  float fa[3][3];
  for (int j = 0; j < 3; ++j)
    for (int r = 0; r < 3; ++r) fa[j][r] = (float)ax[j][r];
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int i = b; i < e; ++i)
    for (int k = 0; k < 3; ++k) {
      const double* p = &V[3 * (size_t)T[3 * (size_t)perm[i] + k]];
      for (int j = 0; j < 3; ++j) {
        const double s = fa[j][0] * p[0] + fa[j][1] * p[1] + fa[j][2] * p[2];
        lo[j] = std::min(lo[j], s);
        hi[j] = std::max(hi[j], s);
      }
    }
  // centre in world coordinates from the FP32 axes, rounded to FP32
  double mid[3];
  for (int j = 0; j < 3; ++j) mid[j] = 0.5 * (lo[j] + hi[j]);
  float fc[3];
  for (int r = 0; r < 3; ++r) fc[r] = (float)(fa[0][r] * mid[0] + fa[1][r] * mid[1] + fa[2][r] * mid[2]);
  // extents measured against the stored centre and axes, rounded up
  double ext[3] = {0, 0, 0};
  for (int i = b; i < e; ++i)
    for (int k = 0; k < 3; ++k) {
      const double* p = &V[3 * (size_t)T[3 * (size_t)perm[i] + k]];
      const double d[3] = {p[0] - fc[0], p[1] - fc[1], p[2] - fc[2]};
      for (int j = 0; j < 3; ++j) ext[j] = std::max(ext[j], std::abs(fa[j][0] * d[0] + fa[j][1] * d[1] + fa[j][2] * d[2]));
    }
  for (int r = 0; r < 3; ++r)
    for (int j = 0; j < 3; ++j) out.axis[3 * r + j] = fa[j][r];
  for (int r = 0; r < 3; ++r) out.center[r] = fc[r];
  for (int j = 0; j < 3; ++j) out.extent[j] = std::nextafter((float)(ext[j] * (1.0 + 1e-6) + 1e-9), INFINITY);
  int longest = 0;
  for (int j = 1; j < 3; ++j)
    if (hi[j] - lo[j] > hi[longest] - lo[longest]) longest = j;
  return longest;
}

}  // namespace

int build_obb_bvh(const float* vertices_xyz, uint32_t nv, const int32_t* tris, uint32_t nt,
                  std::vector<MeshNodeRec>& nodes, std::vector<float>& tri_xyzw) {
  if (nt == 0 || nv == 0) return -1;
  for (uint64_t i = 0; i < 3ull * nt; ++i)
    if (tris[i] < 0 || (uint32_t)tris[i] >= nv) return -2;
  std::vector<double> V(3 * (size_t)nv);
  for (size_t i = 0; i < V.size(); ++i) V[i] = vertices_xyz[i];
  std::vector<int32_t> T(tris, tris + 3 * (size_t)nt);
  tri_xyzw.assign(12 * (size_t)nt, 0.f);
  for (uint32_t t = 0; t < nt; ++t)
    for (int k = 0; k < 3; ++k)
      for (int c = 0; c < 3; ++c) tri_xyzw[12 * (size_t)t + 4 * k + c] = vertices_xyz[3 * (size_t)T[3 * t + k] + c];
  // centroids from the FP32 vertices
  std::vector<double> cen(3 * (size_t)nt);
  for (uint32_t t = 0; t < nt; ++t)
    for (int c = 0; c < 3; ++c)
      cen[3 * t + c] = ((double)vertices_xyz[3 * (size_t)T[3 * t] + c] + vertices_xyz[3 * (size_t)T[3 * t + 1] + c] +
                        vertices_xyz[3 * (size_t)T[3 * t + 2] + c]) / 3.0;
  std::vector<int> perm(nt);
  for (uint32_t i = 0; i < nt; ++i) perm[i] = (int)i;
  nodes.assign(2 * (size_t)nt - 1, MeshNodeRec{});
  int next = 1;
  std::vector<Work> stack;
  stack.push_back({0, 0, (int)nt});
  while (!stack.empty()) {
    const Work w = stack.back();
    stack.pop_back();
    MeshNodeRec& node = nodes[w.node];
    const int longest = fit_node(V, T, perm, w.begin, w.end, node);
    if (w.end - w.begin == 1) {
      node.child = -(perm[w.begin] + 1);
      continue;
    }
    const float* a = &node.axis[0];
    auto proj = [&](int t) {
      return a[longest] * cen[3 * t] + a[3 + longest] * cen[3 * t + 1] + a[6 + longest] * cen[3 * t + 2];
    };
    double m = 0;
    for (int i = w.begin; i < w.end; ++i) m += proj(perm[i]);
    m /= (w.end - w.begin);
    int mid = (int)(std::partition(perm.begin() + w.begin, perm.begin() + w.end, [&](int t) { return proj(t) < m; }) -
                    perm.begin());
    if (mid == w.begin || mid == w.end) {  // all centroids on one side: split at the median
      mid = (w.begin + w.end) / 2;
      std::nth_element(perm.begin() + w.begin, perm.begin() + mid, perm.begin() + w.end,
                       [&](int x, int y) { return proj(x) < proj(y); });
    }
    node.child = next;
    stack.push_back({next + 1, mid, w.end});
    stack.push_back({next, w.begin, mid});
    next += 2;
  }
  return 0;
}

}  // namespace fclg
