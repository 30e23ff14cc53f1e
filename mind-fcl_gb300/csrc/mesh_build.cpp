// Host-side BVH build for triangle meshes: the reference's own OBBRSS tree.
//
// Reproduces BVHModel<OBBRSS<double>>::endModel on a triangle mesh
// (geometry/bvh/BVH_model-inl.h:403-440 buildTreeIterativeImpl, :450-570
// iterativeBuildTree) in FP64 with the reference's operation order, so the
// tree — node slots, children, leaf triangles, and each node's |extent|^2
// that decides which side the traversal descends — is the reference's,
// bit for bit.  The traversal order of a mesh-mesh query, and therefore which
// contacts a capped request keeps, depends on exactly these.
//
//   fit (BV_fitter-inl.h:323-345, OBB half of FitImpl<S, OBBRSS<S>>):
//     covariance of the node's triangle vertices (getCovariance,
//     math/geometry-inl.h:712-767), eigenvectors by eigen_old's Jacobi
//     sweeps (:236-337), axes by axisFromEigen (:339-366: largest, middle,
//     their cross product), centre and half extents from the vertices'
//     projections (getExtentAndCenter_mesh, :147-182);
//   split (BV_splitter-inl.h, default SPLIT_METHOD_MEAN for OBBRSS):
//     split vector = the first box axis (:449-454), split value = the mean
//     of the triangle centroids projected on it (computeSplitValue_mean,
//     :464-506); a triangle stays right when its centroid projects above the
//     value (ApplyImpl<OBBRSS>, :411-415), otherwise it is swapped to the
//     left block; an empty side falls back to half / half;
//   order: a node's children take the next two slots (left, right) and the
//     left subtree is built first (the task stack pushes right, then left).
//
// The GPU keeps an FP32 copy of each box: the FP64 axes and centre rounded to
// FP32 and the extents re-measured in FP64 against those rounded values over
// the node's vertices and rounded up, so every stored box contains all of
// its triangles exactly.  The traversal's FP32 box test is conservative on
// top of that, so it never drops a node pair whose subtree holds a
// colliding triangle pair.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

#include "mesh_build.h"

namespace fclg {

namespace {

struct Obb64 {
  double ax[3][3];  // ax[j] = box axis j (the reference's axis.col(j))
  double to[3];
  double ext[3];
};

using Tri = const int32_t*;

// Sum of coordinates and second moments over the block's vertices, in the
// reference's accumulation order.
void covariance(const double* V, const int32_t* T, const uint32_t* idx, int n, double M[3][3]) {
  double s1[3] = {0, 0, 0};
  double xx = 0, yy = 0, zz = 0, xy = 0, xz = 0, yz = 0;
  for (int i = 0; i < n; ++i) {
    const Tri t = T + 3 * (size_t)idx[i];
    const double* a = V + 3 * (size_t)t[0];
    const double* b = V + 3 * (size_t)t[1];
    const double* c = V + 3 * (size_t)t[2];
    for (int k = 0; k < 3; ++k) s1[k] += (a[k] + b[k]) + c[k];
    xx += (a[0] * a[0] + b[0] * b[0] + c[0] * c[0]);
    yy += (a[1] * a[1] + b[1] * b[1] + c[1] * c[1]);
    zz += (a[2] * a[2] + b[2] * b[2] + c[2] * c[2]);
    xy += (a[0] * a[1] + b[0] * b[1] + c[0] * c[1]);
    xz += (a[0] * a[2] + b[0] * b[2] + c[0] * c[2]);
    yz += (a[1] * a[2] + b[1] * b[2] + c[1] * c[2]);
  }
  const int np = 3 * n;
  M[0][0] = xx - s1[0] * s1[0] / np;
  M[1][1] = yy - s1[1] * s1[1] / np;
  M[2][2] = zz - s1[2] * s1[2] / np;
  M[0][1] = M[1][0] = xy - s1[0] * s1[1] / np;
  M[1][2] = M[2][1] = yz - s1[1] * s1[2] / np;
  M[0][2] = M[2][0] = xz - s1[0] * s1[2] / np;
}

// Jacobi eigen-decomposition with the reference's threshold schedule and
// update formulas.  On return vec[k] is the eigenvector of val[k] (column k of
// the accumulated rotation).  When 50 sweeps leave an off-diagonal entry the
// outputs keep their zero initial values, as the reference's do.
void jacobi_eigen(const double Min[3][3], double val[3], double vec[3][3]) {
  double a[3][3];
  std::memcpy(a, Min, sizeof a);
  double rot[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  double base[3], acc[3], diag[3];
  for (int p = 0; p < 3; ++p) {
    base[p] = diag[p] = a[p][p];
    acc[p] = 0;
  }
  for (int k = 0; k < 3; ++k) {
    val[k] = 0;
    for (int j = 0; j < 3; ++j) vec[k][j] = 0;
  }
  for (int sweep = 0; sweep < 50; ++sweep) {
    double off = 0;
    for (int p = 0; p < 3; ++p)
      for (int q = p + 1; q < 3; ++q) off += std::abs(a[p][q]);
    if (off == 0.0) {
      for (int k = 0; k < 3; ++k) {
        val[k] = diag[k];
        for (int j = 0; j < 3; ++j) vec[k][j] = rot[j][k];
      }
      return;
    }
    const double thresh = sweep < 3 ? 0.2 * off / 9 : 0.0;
    for (int p = 0; p < 3; ++p) {
      for (int q = p + 1; q < 3; ++q) {
        const double g = 100.0 * std::abs(a[p][q]);
        if (sweep > 3 && std::abs(diag[p]) + g == std::abs(diag[p]) && std::abs(diag[q]) + g == std::abs(diag[q])) {
          a[p][q] = 0.0;
          continue;
        }
        if (!(std::abs(a[p][q]) > thresh)) continue;
        double h = diag[q] - diag[p];
        double t;
        if (std::abs(h) + g == std::abs(h)) {
          t = a[p][q] / h;
        } else {
          const double theta = 0.5 * h / a[p][q];
          t = 1.0 / (std::abs(theta) + std::sqrt(1.0 + theta * theta));
          if (theta < 0.0) t = -t;
        }
        const double c = 1.0 / std::sqrt(1 + t * t), s = t * c, tau = s / (1.0 + c);
        h = t * a[p][q];
        acc[p] -= h;
        acc[q] += h;
        diag[p] -= h;
        diag[q] += h;
        a[p][q] = 0.0;
        auto turn = [&](double& x, double& y) {
          const double gx = x, hy = y;
          x = gx - s * (hy + gx * tau);
          y = hy + s * (gx - hy * tau);
        };
        for (int j = 0; j < p; ++j) turn(a[j][p], a[j][q]);
        for (int j = p + 1; j < q; ++j) turn(a[p][j], a[j][q]);
        for (int j = q + 1; j < 3; ++j) turn(a[p][j], a[q][j]);
        for (int j = 0; j < 3; ++j) turn(rot[j][p], rot[j][q]);
      }
    }
    for (int p = 0; p < 3; ++p) {
      base[p] += acc[p];
      diag[p] = base[p];
      acc[p] = 0.0;
    }
  }
}

void fit_obb(const double* V, const int32_t* T, const uint32_t* idx, int n, Obb64& o) {
  double M[3][3], val[3], vec[3][3];
  covariance(V, T, idx, n, M);
  jacobi_eigen(M, val, vec);
  // largest and middle eigenvalue (ties resolved as the reference does)
  int lo, hi, mid;
  if (val[0] > val[1]) {
    hi = 0;
    lo = 1;
  } else {
    lo = 0;
    hi = 1;
  }
  if (val[2] < val[lo]) {
    mid = lo;
    lo = 2;
  } else if (val[2] > val[hi]) {
    mid = hi;
    hi = 2;
  } else {
    mid = 2;
  }
  for (int k = 0; k < 3; ++k) {
    o.ax[0][k] = vec[hi][k];
    o.ax[1][k] = vec[mid][k];
  }
  const double* u = o.ax[0];
  const double* v = o.ax[1];
  o.ax[2][0] = u[1] * v[2] - u[2] * v[1];
  o.ax[2][1] = u[2] * v[0] - u[0] * v[2];
  o.ax[2][2] = u[0] * v[1] - u[1] * v[0];
  const double big = std::numeric_limits<double>::max();
  double mn[3] = {big, big, big}, mx[3] = {-big, -big, -big};
  for (int i = 0; i < n; ++i) {
    const Tri t = T + 3 * (size_t)idx[i];
    for (int j = 0; j < 3; ++j) {
      const double* p = V + 3 * (size_t)t[j];
      for (int k = 0; k < 3; ++k) {
        const double s = (o.ax[k][0] * p[0] + o.ax[k][1] * p[1]) + o.ax[k][2] * p[2];
        if (s > mx[k]) mx[k] = s;
        if (s < mn[k]) mn[k] = s;
      }
    }
  }
  double mid3[3];
  for (int k = 0; k < 3; ++k) mid3[k] = (mx[k] + mn[k]) / 2;
  for (int r = 0; r < 3; ++r) o.to[r] = (o.ax[0][r] * mid3[0] + o.ax[1][r] * mid3[1]) + o.ax[2][r] * mid3[2];
  for (int k = 0; k < 3; ++k) o.ext[k] = (mx[k] - mn[k]) / 2;
}

// FP32 copy of a box that contains the block's vertices exactly.
void store_node(const double* V, const int32_t* T, const uint32_t* idx, int n, const Obb64& o, MeshNodeRec& out) {
  float fa[3][3], fc[3];
  for (int j = 0; j < 3; ++j)
    for (int r = 0; r < 3; ++r) fa[j][r] = (float)o.ax[j][r];
  for (int r = 0; r < 3; ++r) fc[r] = (float)o.to[r];
  double ext[3] = {0, 0, 0};
  for (int i = 0; i < n; ++i) {
    const Tri t = T + 3 * (size_t)idx[i];
    for (int k = 0; k < 3; ++k) {
      const double* p = V + 3 * (size_t)t[k];
      const double d[3] = {p[0] - fc[0], p[1] - fc[1], p[2] - fc[2]};
      for (int j = 0; j < 3; ++j)
        ext[j] = std::max(ext[j], std::abs((double)fa[j][0] * d[0] + (double)fa[j][1] * d[1] + (double)fa[j][2] * d[2]));
    }
  }
  for (int r = 0; r < 3; ++r)
    for (int j = 0; j < 3; ++j) out.axis[3 * r + j] = fa[j][r];
  for (int r = 0; r < 3; ++r) out.center[r] = fc[r];
  for (int j = 0; j < 3; ++j) out.extent[j] = std::nextafter((float)(ext[j] * (1.0 + 1e-6) + 1e-9), INFINITY);
}

}  // namespace

int build_obb_bvh(const float* vertices_xyz, uint32_t nv, const int32_t* tris, uint32_t nt,
                  std::vector<MeshNodeRec>& nodes, std::vector<float>& tri_xyzw, std::vector<double>* sizes,
                  uint32_t* depth) {
  if (nt == 0 || nv == 0) return -1;
  for (uint64_t i = 0; i < 3ull * nt; ++i)
    if (tris[i] < 0 || (uint32_t)tris[i] >= nv) return -2;
  std::vector<double> V(3 * (size_t)nv);
  for (size_t i = 0; i < V.size(); ++i) V[i] = vertices_xyz[i];
  const int32_t* T = tris;
  tri_xyzw.assign(12 * (size_t)nt, 0.f);
  for (uint32_t t = 0; t < nt; ++t)
    for (int k = 0; k < 3; ++k)
      for (int c = 0; c < 3; ++c) tri_xyzw[12 * (size_t)t + 4 * k + c] = vertices_xyz[3 * (size_t)T[3 * t + k] + c];
  std::vector<uint32_t> prim(nt);
  for (uint32_t i = 0; i < nt; ++i) prim[i] = i;
  const size_t n_nodes = 2 * (size_t)nt - 1;
  nodes.assign(n_nodes, MeshNodeRec{});
  if (sizes) sizes->assign(n_nodes, 0.0);
  std::vector<uint32_t> level(n_nodes, 0);
  uint32_t max_level = 0;
  struct Task {
    uint32_t node;
    int first, count;
  };
  std::vector<Task> tasks;
  tasks.push_back({0, 0, (int)nt});
  size_t next = 1;
  while (!tasks.empty()) {
    const Task task = tasks.back();
    tasks.pop_back();
    uint32_t* blk = prim.data() + task.first;
    Obb64 o;
    fit_obb(V.data(), T, blk, task.count, o);
    MeshNodeRec& rec = nodes[task.node];
    store_node(V.data(), T, blk, task.count, o, rec);
    if (sizes) (*sizes)[task.node] = (o.ext[0] * o.ext[0] + o.ext[1] * o.ext[1]) + o.ext[2] * o.ext[2];
    max_level = std::max(max_level, level[task.node]);
    if (task.count == 1) {
      rec.child = -((int32_t)blk[0] + 1);
      continue;
    }
    const double axis0[3] = {o.ax[0][0], o.ax[0][1], o.ax[0][2]};
    double csum[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < task.count; ++i) {
      const Tri t = T + 3 * (size_t)blk[i];
      const double* a = &V[3 * (size_t)t[0]];
      const double* b = &V[3 * (size_t)t[1]];
      const double* c = &V[3 * (size_t)t[2]];
      for (int k = 0; k < 3; ++k) csum[k] += ((a[k] + b[k]) + c[k]) / 3;
    }
    const double split = ((csum[0] * axis0[0] + csum[1] * axis0[1]) + csum[2] * axis0[2]) / task.count;
    int n_left = 0;
    for (int i = 0; i < task.count; ++i) {
      const Tri t = T + 3 * (size_t)blk[i];
      const double* a = &V[3 * (size_t)t[0]];
      const double* b = &V[3 * (size_t)t[1]];
      const double* c = &V[3 * (size_t)t[2]];
      double g[3];
      for (int k = 0; k < 3; ++k) g[k] = ((a[k] + b[k]) + c[k]) / 3.0;
      const bool right = ((axis0[0] * g[0] + axis0[1] * g[1]) + axis0[2] * g[2]) > split;
      if (!right) std::swap(blk[i], blk[n_left++]);
    }
    if (n_left == 0 || n_left == task.count) n_left = task.count / 2;
    const uint32_t left = (uint32_t)next;
    next += 2;
    rec.child = (int32_t)left;
    level[left] = level[left + 1] = level[task.node] + 1;
    tasks.push_back({left + 1, task.first + n_left, task.count - n_left});
    tasks.push_back({left, task.first, n_left});
  }
  if (depth) *depth = max_level;
  return 0;
}

}  // namespace fclg
