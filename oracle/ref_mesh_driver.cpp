// ORACLE — test infrastructure only.
//
// Driver that runs the reference's own mesh and closed-form shape code,
// compiled unmodified through oracle/eigen_shim_full (a general fixed-size
// Eigen subset written for this project):
//   * BVHModel<OBBRSS<double>> built by beginModel / addSubModel / endModel
//     (include/fcl/geometry/bvh/BVH_model-inl.h:136-303, 450-570) with its
//     default mean splitter and OBBRSS fitter (BV_fitter-inl.h:323-345);
//   * OrientedNodeBVHSolver<OBBRSS<double>>::MeshIntersect
//     (include/fcl/narrowphase/detail/traversal/collision/bvh_solver-inl.h:74-164)
//     with the boolean request (no penetration) and a contact cap;
//   * OrientedNodeBVHSolver<OBBRSS<double>>::MeshShapeIntersect
//     (bvh_solver-inl.h:6-72) of such a mesh against a sphere, box, capsule,
//     cylinder or Convex, boolean request with a contact cap;
//   * GJKSolver<double>::shapeIntersect on sphere / box / capsule / cylinder
//     pairs, i.e. the closed-form solvers fcl::collide dispatches to
//     (gjk_solver-inl.h:209-218: sphereSphereIntersect, sphereBoxIntersect,
//     sphereCapsuleIntersect, sphereCylinderIntersect, boxBoxIntersect).
// oracle/build_ref.sh builds it into oracle/_ref/libfcl_ref_mesh.so; it needs
// the reference sources and is therefore only built where they exist.  Tests
// use it to pin the FP64 restatements and to generate golden fixtures.
#include <cstdint>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

#include "fcl/geometry/shape/convex.h"
#include "fcl/narrowphase/detail/shape_pair_intersect.h"
#include "fcl/narrowphase/detail/traversal/collision/bvh_solver.h"

using namespace fcl;

namespace {

using Model = BVHModel<OBBRSS<double>>;

struct Handle {
  Model model;
};

Transform3<double> pose_tf(const double* p) {
  // 12 doubles: rotation row-major, then translation
  Transform3<double> tf = Transform3<double>::Identity();
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) tf.linear()(r, c) = p[3 * r + c];
  tf.translation() = Vector3<double>(p[9], p[10], p[11]);
  return tf;
}

template <class F>
void parallel_for(int n, int threads, F&& f) {
  if (threads <= 1 || n < 2 * threads) {
    f(0, n);
    return;
  }
  std::vector<std::thread> pool;
  const int chunk = (n + threads - 1) / threads;
  for (int t = 0; t < threads; ++t) {
    const int b = t * chunk, e = std::min(n, b + chunk);
    if (b < e) pool.emplace_back([&, b, e] { f(b, e); });
  }
  for (auto& th : pool) th.join();
}

// Shape record of the analytic entry point: type (0 sphere, 1 box, 2 capsule,
// 3 cylinder) and parameters (sphere r; box full sides; capsule / cylinder r,
// full length).
struct AnShape {
  int32_t type;
  double p[3];
};

template <class S1, class S2>
int run_pair(const S1& a, const S2& b, const Transform3<double>& tf1, const Transform3<double>& tf2,
             double* out) {
  detail::GJKSolver<double> solver;
  CollisionPenetrationContactData<double> contacts;
  const bool hit = solver.shapeIntersect(a, tf1, b, tf2, &contacts);
  const int n = hit ? (int)contacts.size() : 0;
  for (int k = 0; k < n && k < 4; ++k) {
    const ContactPoint<double>& c = contacts[k];
    for (int j = 0; j < 3; ++j) {
      out[7 * k + j] = c.normal[j];
      out[7 * k + 3 + j] = c.pos[j];
    }
    out[7 * k + 6] = c.penetration_depth;
  }
  return hit ? (n > 0 ? n : 1) : 0;
}

template <class S1>
int dispatch_b(const S1& a, const AnShape& sb, const Transform3<double>& tf1, const Transform3<double>& tf2,
               double* out) {
  switch (sb.type) {
    case 0: return run_pair(a, Sphere<double>(sb.p[0]), tf1, tf2, out);
    case 1: return run_pair(a, Box<double>(sb.p[0], sb.p[1], sb.p[2]), tf1, tf2, out);
    case 2: return run_pair(a, Capsule<double>(sb.p[0], sb.p[1]), tf1, tf2, out);
    case 3: return run_pair(a, Cylinder<double>(sb.p[0], sb.p[1]), tf1, tf2, out);
  }
  return -1;
}

}  // namespace

extern "C" {

// Builds the reference's OBBRSS tree over nt triangles (indices into nv
// vertices, xyz doubles).  Returns a handle, or null on a build error.
void* refm_build(const double* V, int nv, const int32_t* T, int nt) {
  std::unique_ptr<Handle> h(new Handle);
  std::vector<Vector3<double>> pts(nv);
  for (int i = 0; i < nv; ++i) pts[i] = Vector3<double>(V[3 * i], V[3 * i + 1], V[3 * i + 2]);
  std::vector<MeshSimplex> tris(nt);
  for (int i = 0; i < nt; ++i) tris[i] = MeshSimplex(T[3 * i], T[3 * i + 1], T[3 * i + 2]);
  if (h->model.beginModel() != BVH_OK) return nullptr;
  if (h->model.addSubModel(pts, tris) != BVH_OK) return nullptr;
  if (h->model.endModel() != BVH_OK) return nullptr;
  return h.release();
}

void refm_free(void* h) { delete static_cast<Handle*>(h); }

int refm_num_nodes(void* h) { return static_cast<Handle*>(h)->model.getNumBVs(); }

// Per node: f64[16] = OBB axis (row-major; its columns are the box axes), To,
// extent, size() (= |extent|^2, the traversal's descend key); i32[3] =
// first_child (< 0: leaf of primitive -(first_child + 1)), first_primitive,
// num_primitives.
void refm_export(void* hp, double* f64, int32_t* i32) {
  const Model& m = static_cast<Handle*>(hp)->model;
  for (int i = 0; i < m.getNumBVs(); ++i) {
    const BVNode<OBBRSS<double>>& n = m.getBV(i);
    const OBB<double>& o = n.bv.obb;
    double* d = f64 + 16 * (size_t)i;
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) d[3 * r + c] = o.axis(r, c);
    for (int k = 0; k < 3; ++k) {
      d[9 + k] = o.To[k];
      d[12 + k] = o.extent[k];
    }
    d[15] = n.bv.size();
    i32[3 * (size_t)i] = n.first_child;
    i32[3 * (size_t)i + 1] = n.first_primitive;
    i32[3 * (size_t)i + 2] = n.num_primitives;
  }
}

// MeshIntersect for each pose (mesh a at the identity, mesh b posed by
// poses[i], 12 doubles) with CollisionRequest(cap): counts[i] = the number of
// contacts, pairs[i][k] = (b1, b2) of contact k in the order the reference
// adds them, for k < stride.
int refm_mesh_collide(void* ha, void* hb, const double* poses, int n, int cap, int32_t* counts, int32_t* pairs,
                      int stride, int threads) {
  const Model& a = static_cast<Handle*>(ha)->model;
  const Model& b = static_cast<Handle*>(hb)->model;
  parallel_for(n, threads, [&](int lo, int hi) {
    detail::GJKSolver<double> solver;
    detail::OrientedNodeBVHSolver<OBBRSS<double>> bs(&solver);
    const CollisionRequest<double> req((std::size_t)cap);
    const Transform3<double> tf1 = Transform3<double>::Identity();
    for (int i = lo; i < hi; ++i) {
      CollisionResult<double> res;
      bs.MeshIntersect(&a, &b, tf1, pose_tf(poses + 12 * (size_t)i), req, res);
      counts[i] = (int32_t)res.numContacts();
      for (int k = 0; k < (int)res.numContacts() && k < stride; ++k) {
        pairs[((size_t)i * stride + k) * 2] = (int32_t)res.getContact(k).b1;
        pairs[((size_t)i * stride + k) * 2 + 1] = (int32_t)res.getContact(k).b2;
      }
    }
  });
  return 0;
}

// GJKSolver::shapeIntersect with contacts for shape a at the identity and
// shape b posed by poses[i]; only sphere-sphere / -box / -capsule / -cylinder
// (either order) and box-box are accepted (the closed-form solvers).  out[i]:
// 4 x (normal 3, pos 3, depth); returns per pair (in ret[i]) the contact
// count, 0 when separated, -1 for a pair outside that set.
int refm_analytic(const void* shapes_a, const void* shapes_b, const double* poses, int n, double* out, int32_t* ret,
                  int threads) {
  const AnShape* A = static_cast<const AnShape*>(shapes_a);
  const AnShape* B = static_cast<const AnShape*>(shapes_b);
  parallel_for(n, threads, [&](int lo, int hi) {
    const Transform3<double> tf1 = Transform3<double>::Identity();
    for (int i = lo; i < hi; ++i) {
      const Transform3<double> tf2 = pose_tf(poses + 12 * (size_t)i);
      double* o = out + 28 * (size_t)i;
      std::memset(o, 0, 28 * sizeof(double));
      const AnShape& sa = A[i];
      const AnShape& sb = B[i];
      const bool sphere_pair = sa.type == 0 || sb.type == 0;
      const bool box_box = sa.type == 1 && sb.type == 1;
      if (!sphere_pair && !box_box) {
        ret[i] = -1;
        continue;
      }
      switch (sa.type) {
        case 0: ret[i] = dispatch_b(Sphere<double>(sa.p[0]), sb, tf1, tf2, o); break;
        case 1: ret[i] = dispatch_b(Box<double>(sa.p[0], sa.p[1], sa.p[2]), sb, tf1, tf2, o); break;
        case 2: ret[i] = dispatch_b(Capsule<double>(sa.p[0], sa.p[1]), sb, tf1, tf2, o); break;
        case 3: ret[i] = dispatch_b(Cylinder<double>(sa.p[0], sa.p[1]), sb, tf1, tf2, o); break;
        default: ret[i] = -1;
      }
    }
  });
  return 0;
}

// MeshShapeIntersect for each pose: the mesh at the identity, the shape
// (type 0 sphere, 1 box, 2 capsule, 3 cylinder, 4 convex; params as
// refm_analytic's; a convex's vertices hull_v (nv x 3) and faces in fcl's
// encoding (count, then the vertex indices, per face) posed by poses[i] in
// the mesh frame, with CollisionRequest(cap).  counts[i] = contacts,
// tris[i][k] = triangle (b1) of contact k in the reference's order, k < stride.
int refm_mesh_shape_collide(void* hm, int type, const double* params, const double* hull_v, int nv,
                            const int32_t* faces, int n_faces, int faces_len, const double* poses, int n, int cap,
                            int32_t* counts, int32_t* tris, int stride, int threads) {
  const Model& mesh = static_cast<Handle*>(hm)->model;
  std::shared_ptr<std::vector<Vector3<double>>> cv;
  std::shared_ptr<std::vector<int>> cf;
  if (type == 4) {
    cv = std::make_shared<std::vector<Vector3<double>>>(nv);
    for (int i = 0; i < nv; ++i) (*cv)[i] = Vector3<double>(hull_v[3 * i], hull_v[3 * i + 1], hull_v[3 * i + 2]);
    cf = std::make_shared<std::vector<int>>(faces, faces + faces_len);
  }
  auto body = [&](const auto& shape) {
    parallel_for(n, threads, [&](int lo, int hi) {
      detail::GJKSolver<double> solver;
      detail::OrientedNodeBVHSolver<OBBRSS<double>> bs(&solver);
      const CollisionRequest<double> req((std::size_t)cap);
      const Transform3<double> tf1 = Transform3<double>::Identity();
      for (int i = lo; i < hi; ++i) {
        CollisionResult<double> res;
        bs.MeshShapeIntersect(&mesh, shape, tf1, pose_tf(poses + 12 * (size_t)i), req, res);
        counts[i] = (int32_t)res.numContacts();
        for (int k = 0; k < (int)res.numContacts() && k < stride; ++k)
          tris[(size_t)i * stride + k] = (int32_t)res.getContact(k).b1;
      }
    });
  };
  switch (type) {
    case 0: body(Sphere<double>(params[0])); break;
    case 1: body(Box<double>(params[0], params[1], params[2])); break;
    case 2: body(Capsule<double>(params[0], params[1])); break;
    case 3: body(Cylinder<double>(params[0], params[1])); break;
    case 4: body(Convex<double>(cv, n_faces, cf)); break;
    default: return -1;
  }
  return 0;
}

}  // extern "C"
