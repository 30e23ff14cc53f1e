// fclg_fcl.hpp — the reference's C++ narrowphase API (fcl::collide,
// detail::GJKSolver::shapeSignedDistance, the geometry classes) over the fclg
// C ABI, so C++ callers of mind-fcl can switch by changing a namespace and an
// include.  Header-only C++17; link with libfclg.so.
//
// Mirrors (paths relative to the mind-fcl project root):
//   fcl::collide                       include/fcl/narrowphase/collision.h:54-58
//   CollisionRequest / CollisionResult include/fcl/narrowphase/collision_request.h:50-95,
//                                      collision_result.h:61-93
//   Contact                            include/fcl/narrowphase/contact.h:47-98
//   GJKSolver::shapeSignedDistance     include/fcl/narrowphase/detail/gjk_solver.h:97-100,
//                                      gjk_solver-inl.h:810-863
//   Box / Sphere / Capsule / Cylinder  include/fcl/geometry/shape/{box,sphere,capsule,cylinder}.h
//   Convex                             include/fcl/geometry/shape/convex.h:106-108
//   BVHModel<OBBRSS>                   include/fcl/geometry/bvh/BVH_model.h:103-123
//
// Differences a caller sees:
//   * Transform arguments are templates: any type with linear()(i, j) and
//     translation()(i) — Eigen::Transform / Eigen::Isometry3d as the reference
//     uses, or the small fclg::fcl::Transform3 below (no Eigen needed).
//   * Computation is FP32 on the GPU with FP64 where degenerate (see the
//     library's parity bar); results come back in S.
//   * Each call runs on a per-thread context of device 0 (setDevice() before
//     the first call to change it).  One pair per call is a GPU round trip;
//     BatchQuery runs many pairs per call and is the fast path.
//   * Mesh-mesh and mesh-shape pairs: boolean contacts with triangle indices.
//   * Penetration modes: disabled (boolean), the default GJK/EPA mode, and
//     the MPR directed / incremental minimum-distance modes
//     (useDirectedPenetration / useIncrementalMinimumDistancePenetration,
//     collision_request.h:74-79) for shape pairs.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <iostream>
#include <memory>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "fclg.h"

namespace fclg {
namespace fcl {

template <typename S>
struct Vector3 {
  S v[3] = {S(0), S(0), S(0)};
  Vector3() = default;
  Vector3(S x, S y, S z) : v{x, y, z} {}
  S& operator()(int i) { return v[i]; }
  S operator()(int i) const { return v[i]; }
  S& operator[](int i) { return v[i]; }
  S operator[](int i) const { return v[i]; }
  S x() const { return v[0]; }
  S y() const { return v[1]; }
  S z() const { return v[2]; }
};

template <typename S>
struct Matrix3 {
  S m[9] = {S(1), S(0), S(0), S(0), S(1), S(0), S(0), S(0), S(1)};
  S& operator()(int i, int j) { return m[3 * i + j]; }
  S operator()(int i, int j) const { return m[3 * i + j]; }
};

// Rigid transform (rotation + translation), the subset of Eigen::Isometry3 the
// API reads.
template <typename S>
struct Transform3 {
  Matrix3<S> R;
  Vector3<S> t;
  static Transform3 Identity() { return Transform3(); }
  Matrix3<S>& linear() { return R; }
  const Matrix3<S>& linear() const { return R; }
  Vector3<S>& translation() { return t; }
  const Vector3<S>& translation() const { return t; }
};

enum NODE_TYPE { GEOM_BOX, GEOM_SPHERE, GEOM_CAPSULE, GEOM_CYLINDER, GEOM_CONVEX, BV_OBBRSS };

template <typename S>
class CollisionGeometry {
 public:
  virtual ~CollisionGeometry() = default;
  virtual NODE_TYPE getNodeType() const = 0;
};

template <typename S>
class Box : public CollisionGeometry<S> {
 public:
  Box(S x, S y, S z) : side(x, y, z) {}
  explicit Box(const Vector3<S>& s) : side(s) {}
  Box() : side(S(0), S(0), S(0)) {}
  Vector3<S> side;  // full side lengths, as the reference stores them (box.h:63)
  NODE_TYPE getNodeType() const override { return GEOM_BOX; }
};

template <typename S>
class Sphere : public CollisionGeometry<S> {
 public:
  explicit Sphere(S r) : radius(r) {}
  S radius;
  NODE_TYPE getNodeType() const override { return GEOM_SPHERE; }
};

template <typename S>
class Capsule : public CollisionGeometry<S> {
 public:
  Capsule(S r, S l) : radius(r), lz(l) {}
  S radius, lz;  // lz: full length of the segment along z
  NODE_TYPE getNodeType() const override { return GEOM_CAPSULE; }
};

template <typename S>
class Cylinder : public CollisionGeometry<S> {
 public:
  Cylinder(S r, S l) : radius(r), lz(l) {}
  S radius, lz;
  NODE_TYPE getNodeType() const override { return GEOM_CYLINDER; }
};

// Convex hull given by its vertices (the face encoding is accepted and kept
// for the caller; the support mapping needs only the vertices).
template <typename S>
class Convex : public CollisionGeometry<S> {
 public:
  Convex(const std::shared_ptr<const std::vector<Vector3<S>>>& vertices, int num_faces,
         const std::shared_ptr<const std::vector<int>>& faces, bool throw_if_invalid = false)
      : vertices_(vertices), num_faces_(num_faces), faces_(faces) {
    if (throw_if_invalid && (!vertices_ || vertices_->empty())) throw std::invalid_argument("Convex: no vertices");
  }
  const std::vector<Vector3<S>>& getVertices() const { return *vertices_; }
  int getFaceCount() const { return num_faces_; }
  const std::vector<int>& getFaces() const { return *faces_; }
  NODE_TYPE getNodeType() const override { return GEOM_CONVEX; }

 private:
  std::shared_ptr<const std::vector<Vector3<S>>> vertices_;
  int num_faces_;
  std::shared_ptr<const std::vector<int>> faces_;
};

template <typename S>
struct OBBRSS {
  using Scalar = S;
};

struct Triangle {
  std::size_t vids[3];
  Triangle() : vids{0, 0, 0} {}
  Triangle(std::size_t a, std::size_t b, std::size_t c) : vids{a, b, c} {}
  std::size_t operator[](int i) const { return vids[i]; }
};

namespace detail {
struct MeshHandle {
  fclg_mesh* mesh = nullptr;
  ~MeshHandle() {
    if (mesh) fclg_mesh_destroy(mesh);
  }
};
}  // namespace detail

// Triangle-mesh model with an OBB hierarchy, built on the device's first use
// (mean split, OBB fit by covariance eigenvectors, as BVHModel<OBBRSS>).
template <typename BV>
class BVHModel : public CollisionGeometry<typename BV::Scalar> {
 public:
  using S = typename BV::Scalar;
  int beginModel(int = 0, int = 0) {
    verts_.clear();
    tris_.clear();
    built_.reset();
    return 0;
  }
  int addSubModel(const std::vector<Vector3<S>>& points, const std::vector<Triangle>& triangles) {
    const std::size_t base = verts_.size() / 3;
    for (const auto& p : points)
      for (int i = 0; i < 3; ++i) verts_.push_back((float)p[i]);
    for (const auto& t : triangles)
      for (int i = 0; i < 3; ++i) tris_.push_back((int32_t)(base + t[i]));
    return 0;
  }
  int endModel() { return tris_.empty() ? -1 : 0; }
  NODE_TYPE getNodeType() const override { return BV_OBBRSS; }
  int num_tris() const { return (int)(tris_.size() / 3); }
  // The device mesh of context ctx (created on first use).
  fclg_mesh* device_mesh(fclg_context* ctx) const {
    if (!built_) {
      auto h = std::make_shared<detail::MeshHandle>();
      const int rc = fclg_mesh_create(ctx, verts_.data(), (uint32_t)(verts_.size() / 3), tris_.data(),
                                      (uint32_t)(tris_.size() / 3), &h->mesh);
      if (rc != FCLG_OK) throw std::runtime_error(std::string("fclg_mesh_create: ") + fclg_last_error(ctx));
      built_ = h;
    }
    return built_->mesh;
  }

 private:
  std::vector<float> verts_;
  std::vector<int32_t> tris_;
  mutable std::shared_ptr<detail::MeshHandle> built_;
};

template <typename S>
struct Contact {
  const CollisionGeometry<S>* o1 = nullptr;
  const CollisionGeometry<S>* o2 = nullptr;
  intptr_t b1 = -1, b2 = -1;   // triangle indices for meshes, -1 for shapes
  Vector3<S> normal;           // escape direction of o2, world frame: normalize(p1 - p2)
  Vector3<S> pos;              // world frame, 0.5 (p1 + p2)
  S penetration_depth = S(0);
  Contact() = default;
  Contact(const CollisionGeometry<S>* a, const CollisionGeometry<S>* b, int i, int j) : o1(a), o2(b), b1(i), b2(j) {}
};

template <typename S>
class CollisionRequest {
 public:
  CollisionRequest() : CollisionRequest(1) {}
  explicit CollisionRequest(std::size_t n_max_contacts) : num_max_contacts_(n_max_contacts) {}
  void disablePenetration() { penetration_ = false; mode_ = 0; }
  void useDefaultPenetration() { penetration_ = true; mode_ = 0; }
  // MPR penetration along (directed) or starting from (incremental) shape 2's
  // escape direction in the world frame (collision_penetration-inl.h:106-250)
  void useDirectedPenetration(const Vector3<S>& shape2_escape_direction_in_world) {
    penetration_ = true;
    mode_ = 1;
    prior_ = shape2_escape_direction_in_world;
  }
  void useIncrementalMinimumDistancePenetration(const Vector3<S>& shape2_escape_direction_in_world_hint) {
    penetration_ = true;
    mode_ = 2;
    prior_ = shape2_escape_direction_in_world_hint;
  }
  bool isPenetrationEnabled() const { return penetration_; }
  int mprPenetrationMode() const { return mode_; }  // 0 none, 1 directed, 2 incremental
  const Vector3<S>& priorPenetrationDirection() const { return prior_; }
  std::size_t maxNumContacts() const { return num_max_contacts_; }
  void setMaxContactCount(std::size_t n) { num_max_contacts_ = n; }
  void setBinaryCollisionTolerance(S t) { binary_tol_ = t; }
  void setPenetrationDistanceTolerance(S t) { distance_tol_ = t; }
  S binaryCollisionTolerance() const { return binary_tol_; }
  S distanceTolerance() const { return distance_tol_; }

 private:
  std::size_t num_max_contacts_;
  bool penetration_ = false;
  int mode_ = 0;
  Vector3<S> prior_;
  S binary_tol_ = S(1e-6), distance_tol_ = S(1e-6);
};

template <typename S>
class CollisionResult {
 public:
  void addContact(const Contact<S>& c) { contacts_.push_back(c); }
  std::size_t numContacts() const { return contacts_.size(); }
  bool isCollision() const { return !contacts_.empty(); }
  const Contact<S>& getContact(std::size_t i) const { return contacts_.at(i); }
  const std::vector<Contact<S>>& getContacts() const { return contacts_; }
  std::vector<Contact<S>>& getContacts() { return contacts_; }
  void clear() { contacts_.clear(); }

 private:
  std::vector<Contact<S>> contacts_;
};

// ---- translational continuous collision (narrowphase/detail/ccd/) --------
// TranslationalDisplacement and Interval (ccd_typedef.h:11-37).
template <typename S>
struct TranslationalDisplacement {
  Vector3<S> unit_axis_in_shape1;
  S scalar_displacement = S(0);
};

template <typename S>
struct Interval {
  S lower_bound = S(-1);
  S upper_bound = S(-1);
};

// TimeOfCollisionRequestType and ContinuousCollisionRequest (ccd_request.h).
enum class TimeOfCollisionRequestType { kNotRequested, kBoxApproximate, kOneTocSample };

template <typename S>
struct ContinuousCollisionRequest {
  TimeOfCollisionRequestType request_type = TimeOfCollisionRequestType::kNotRequested;
  std::size_t num_max_contacts = 1;
  S zero_movement_tolerance = S(1e-4);
  S gjk_tolerance = S(1e-6);
  int max_gjk_iterations = 128;
};

// ContinuousCollisionContact / ContinuousCollisionResult (ccd_contact.h,
// ccd_result.h): shape pairs give at most one contact, b1 = b2 = -1.
template <typename S>
struct ContinuousCollisionContact {
  const CollisionGeometry<S>* o1 = nullptr;
  const CollisionGeometry<S>* o2 = nullptr;
  int b1 = -1, b2 = -1;
  Interval<S> toc;
};

template <typename S>
class ContinuousCollisionResult {
 public:
  void AddContact(const ContinuousCollisionContact<S>& c) { contacts_.push_back(c); }
  void ClearContact() { contacts_.clear(); }
  std::size_t num_contacts() const { return contacts_.size(); }
  const std::vector<ContinuousCollisionContact<S>>& raw_contacts() const { return contacts_; }
  bool TerminationConditionSatisfied(std::size_t n_max_contacts) const { return contacts_.size() >= n_max_contacts; }

 private:
  std::vector<ContinuousCollisionContact<S>> contacts_;
};

namespace detail {

// Per-thread fclg context (a context is single-threaded, like the reference's per-call solver).
inline int& device_slot() {
  thread_local int device = 0;
  return device;
}

inline fclg_context* thread_context() {
  struct Holder {
    fclg_context* ctx = nullptr;
    ~Holder() {
      if (ctx) fclg_destroy(ctx);
    }
  };
  thread_local Holder h;
  if (!h.ctx) {
    const int rc = fclg_create(&h.ctx, device_slot());
    if (rc != FCLG_OK) throw std::runtime_error("fclg_create failed (" + std::to_string(rc) + ")");
  }
  return h.ctx;
}

inline void check(fclg_context* ctx, int rc, const char* what) {
  if (rc != FCLG_OK) throw std::runtime_error(std::string(what) + ": " + fclg_last_error(ctx));
}

// Appends the fclg_shape record (and convex vertices) of g.
template <typename S>
void encode_shape(const CollisionGeometry<S>* g, std::vector<fclg_shape>& shapes, std::vector<float>& verts) {
  fclg_shape s{};
  switch (g->getNodeType()) {
    case GEOM_BOX: {
      const auto* b = static_cast<const Box<S>*>(g);
      s.type = FCLG_BOX;
      for (int i = 0; i < 3; ++i) s.param[i] = (float)b->side[i];
      break;
    }
    case GEOM_SPHERE:
      s.type = FCLG_SPHERE;
      s.param[0] = (float)static_cast<const Sphere<S>*>(g)->radius;
      break;
    case GEOM_CAPSULE:
      s.type = FCLG_CAPSULE;
      s.param[0] = (float)static_cast<const Capsule<S>*>(g)->radius;
      s.param[1] = (float)static_cast<const Capsule<S>*>(g)->lz;
      break;
    case GEOM_CYLINDER:
      s.type = FCLG_CYLINDER;
      s.param[0] = (float)static_cast<const Cylinder<S>*>(g)->radius;
      s.param[1] = (float)static_cast<const Cylinder<S>*>(g)->lz;
      break;
    case GEOM_CONVEX: {
      const auto& v = static_cast<const Convex<S>*>(g)->getVertices();
      s.type = FCLG_CONVEX;
      s.vert_offset = (uint32_t)(verts.size() / 4);
      s.vert_count = (uint32_t)v.size();
      double c[3] = {0, 0, 0}, r2 = 0;
      for (const auto& p : v) {
        for (int i = 0; i < 3; ++i) {
          verts.push_back((float)p[i]);
          c[i] += (double)p[i];
        }
        verts.push_back(0.f);
        r2 = std::max(r2, (double)p[0] * p[0] + (double)p[1] * p[1] + (double)p[2] * p[2]);
      }
      for (int i = 0; i < 3; ++i) s.param[i] = v.empty() ? 0.f : (float)(c[i] / (double)v.size());
      s.param[3] = (float)std::sqrt(r2);
      break;
    }
    default:
      throw std::invalid_argument("fclg: unsupported geometry in a shape query");
  }
  shapes.push_back(s);
}

// Pose of tf2 in tf1's frame: R = R1^T R2, t = R1^T (t2 - t1) (MinkowskiDiff::toshape0).
template <typename TF1, typename TF2>
void relative_pose(const TF1& tf1, const TF2& tf2, fclg_pair& p) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double a = 0;
      for (int k = 0; k < 3; ++k) a += (double)tf1.linear()(k, i) * (double)tf2.linear()(k, j);
      p.rot[3 * i + j] = (float)a;
    }
  for (int i = 0; i < 3; ++i) {
    double a = 0;
    for (int k = 0; k < 3; ++k)
      a += (double)tf1.linear()(k, i) * ((double)tf2.translation()(k) - (double)tf1.translation()(k));
    p.trans[i] = (float)a;
  }
}

// x in tf's frame -> world
template <typename S, typename TF>
Vector3<S> to_world(const TF& tf, const float* x) {
  Vector3<S> w;
  for (int i = 0; i < 3; ++i) {
    double a = (double)tf.translation()(i);
    for (int k = 0; k < 3; ++k) a += (double)tf.linear()(i, k) * (double)x[k];
    w[i] = (S)a;
  }
  return w;
}
template <typename S, typename TF>
Vector3<S> rotate(const TF& tf, const float* x) {
  Vector3<S> w;
  for (int i = 0; i < 3; ++i) {
    double a = 0;
    for (int k = 0; k < 3; ++k) a += (double)tf.linear()(i, k) * (double)x[k];
    w[i] = (S)a;
  }
  return w;
}

inline fclg_request make_request(uint32_t flags, double gjk_tol, double epa_tol) {
  fclg_request r{};
  r.flags = flags;
  r.gjk_tolerance = (float)gjk_tol;
  r.epa_tolerance = (float)epa_tol;
  return r;
}

}  // namespace detail

inline void setDevice(int device) { detail::device_slot() = device; }

// Many shape pairs per call: the fast path.  Geometries are uploaded once per
// run (deduplicated by address); poses are relative, computed on the host in
// FP64.
template <typename S>
class BatchQuery {
 public:
  template <typename TF1, typename TF2>
  std::size_t add(const CollisionGeometry<S>* o1, const TF1& tf1, const CollisionGeometry<S>* o2, const TF2& tf2) {
    fclg_pair p{};
    p.shape_a = index_of(o1);
    p.shape_b = index_of(o2);
    detail::relative_pose(tf1, tf2, p);
    pairs_.push_back(p);
    frames_.push_back(Frame{});
    Frame& f = frames_.back();
    for (int i = 0; i < 3; ++i) {
      f.t[i] = (double)tf1.translation()(i);
      for (int k = 0; k < 3; ++k) f.R[3 * i + k] = (double)tf1.linear()(i, k);
    }
    geoms_.push_back({o1, o2});
    return pairs_.size() - 1;
  }
  std::size_t size() const { return pairs_.size(); }

  // shapeSignedDistance per pair: ok, distance, witness points in the world frame.
  struct SignedDistance {
    bool ok;
    S distance;
    Vector3<S> p1, p2;
    int status;
  };
  std::vector<SignedDistance> signedDistance(S tolerance = S(1e-6)) {
    std::vector<fclg_result> r = run(true, detail::make_request(0, (double)tolerance, (double)tolerance));
    std::vector<SignedDistance> out(r.size());
    for (std::size_t i = 0; i < r.size(); ++i) {
      out[i].ok = r[i].ok != 0;
      out[i].distance = (S)r[i].distance;
      out[i].p1 = frames_[i].world(r[i].p_a);
      out[i].p2 = frames_[i].world(r[i].p_b);
      out[i].status = r[i].status;
    }
    return out;
  }

  // fcl::collide per pair (one contact per colliding pair with penetration).
  std::vector<CollisionResult<S>> collide(const CollisionRequest<S>& req) {
    if (req.mprPenetrationMode() != 0) return collide_mpr(req);
    const uint32_t flags = req.isPenetrationEnabled() ? 0u : (uint32_t)FCLG_REQ_BOOLEAN_ONLY;
    std::vector<fclg_result> r = run(false, detail::make_request(flags, (double)req.binaryCollisionTolerance(),
                                                                 (double)req.distanceTolerance()));
    std::vector<CollisionResult<S>> out(r.size());
    for (std::size_t i = 0; i < r.size(); ++i) {
      if (!r[i].collide || req.maxNumContacts() == 0) continue;
      Contact<S> c(geoms_[i].first, geoms_[i].second, -1, -1);
      if (req.isPenetrationEnabled() && r[i].ok) {
        c.normal = frames_[i].rot(r[i].normal);
        const float mid[3] = {0.5f * (r[i].p_a[0] + r[i].p_b[0]), 0.5f * (r[i].p_a[1] + r[i].p_b[1]),
                              0.5f * (r[i].p_a[2] + r[i].p_b[2])};
        c.pos = frames_[i].world(mid);
        c.penetration_depth = (S)(-r[i].distance);
      }
      out[i].addContact(c);
    }
    return out;
  }

  // The MPR penetration modes (collisionPenetrationMPR): every colliding pair
  // gets a contact; depth -1, position 0 and the given direction as normal
  // where the MPR run failed, as the reference reports it.
  std::vector<CollisionResult<S>> collide_mpr(const CollisionRequest<S>& req) {
    std::vector<CollisionResult<S>> out(pairs_.size());
    if (pairs_.empty()) return out;
    const Vector3<S>& dw = req.priorPenetrationDirection();
    std::vector<float> dirs(3 * pairs_.size());
    for (std::size_t i = 0; i < pairs_.size(); ++i) {
      const double* R = frames_[i].R;  // direction in shape 1's frame: R^T d
      double a[3];
      for (int k = 0; k < 3; ++k)
        a[k] = R[k] * (double)dw[0] + R[3 + k] * (double)dw[1] + R[6 + k] * (double)dw[2];
      const double l = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
      for (int k = 0; k < 3; ++k) dirs[3 * i + k] = (float)(l > 0 ? a[k] / l : a[k]);
    }
    fclg_request r = detail::make_request(req.mprPenetrationMode() == 2 ? (uint32_t)FCLG_REQ_INCREMENTAL : 0u,
                                          (double)req.binaryCollisionTolerance(), (double)req.distanceTolerance());
    std::vector<fclg_result> res(pairs_.size());
    fclg_context* ctx = detail::thread_context();
    detail::check(ctx, fclg_set_shapes(ctx, shapes_.data(), (uint32_t)shapes_.size(), verts_.data(), verts_.size() / 4),
                  "fclg_set_shapes");
    detail::check(ctx, fclg_collide_directed(ctx, pairs_.data(), (uint32_t)pairs_.size(), dirs.data(), &r, res.data()),
                  "fclg_collide_directed");
    for (std::size_t i = 0; i < res.size(); ++i) {
      if (!res[i].collide || req.maxNumContacts() == 0) continue;
      Contact<S> c(geoms_[i].first, geoms_[i].second, -1, -1);
      if (res[i].ok) {
        c.normal = frames_[i].rot(res[i].normal);
        const float mid[3] = {0.5f * (res[i].p_a[0] + res[i].p_b[0]), 0.5f * (res[i].p_a[1] + res[i].p_b[1]),
                              0.5f * (res[i].p_a[2] + res[i].p_b[2])};
        c.pos = frames_[i].world(mid);
        c.penetration_depth = (S)(-res[i].distance);
      } else {
        c.normal = dw;
        c.pos = Vector3<S>(S(0), S(0), S(0));
        c.penetration_depth = S(-1);
      }
      out[i].addContact(c);
    }
    return out;
  }

  // fcl::translational_ccd per pair: shape 1 of pair i moving along
  // displacement[i] (unit axis in its own frame) against shape 2.
  std::vector<ContinuousCollisionResult<S>> translationalCcd(
      const std::vector<TranslationalDisplacement<S>>& displacement, const ContinuousCollisionRequest<S>& req) {
    std::vector<ContinuousCollisionResult<S>> out(pairs_.size());
    if (pairs_.empty() || req.num_max_contacts == 0) return out;
    if (displacement.size() != pairs_.size()) throw std::invalid_argument("one displacement per pair");
    std::vector<fclg_displacement> disp(pairs_.size());
    for (std::size_t i = 0; i < pairs_.size(); ++i) {
      for (int k = 0; k < 3; ++k) disp[i].axis[k] = (float)displacement[i].unit_axis_in_shape1[k];
      disp[i].distance = (float)displacement[i].scalar_displacement;
    }
    fclg_ccd_request r{};
    r.toc_type = req.request_type == TimeOfCollisionRequestType::kBoxApproximate ? (uint32_t)FCLG_TOC_BOX
                 : req.request_type == TimeOfCollisionRequestType::kOneTocSample ? (uint32_t)FCLG_TOC_SAMPLE
                                                                                  : (uint32_t)FCLG_TOC_NONE;
    r.max_gjk_iterations = req.max_gjk_iterations;
    r.gjk_tolerance = (float)req.gjk_tolerance;
    r.zero_movement_tolerance = (double)req.zero_movement_tolerance;
    std::vector<fclg_ccd_result> res(pairs_.size());
    fclg_context* ctx = detail::thread_context();
    detail::check(ctx, fclg_set_shapes(ctx, shapes_.data(), (uint32_t)shapes_.size(), verts_.data(), verts_.size() / 4),
                  "fclg_set_shapes");
    detail::check(ctx, fclg_translational_ccd(ctx, pairs_.data(), (uint32_t)pairs_.size(), disp.data(), &r, res.data()),
                  "fclg_translational_ccd");
    for (std::size_t i = 0; i < res.size(); ++i) {
      if (!res[i].collide) continue;
      ContinuousCollisionContact<S> c;
      c.o1 = geoms_[i].first;
      c.o2 = geoms_[i].second;
      c.toc.lower_bound = (S)res[i].toc_lower;
      c.toc.upper_bound = (S)res[i].toc_upper;
      out[i].AddContact(c);
    }
    return out;
  }

  void clear() {
    pairs_.clear();
    frames_.clear();
    geoms_.clear();
    shapes_.clear();
    verts_.clear();
    index_.clear();
  }

 private:
  struct Frame {
    double R[9], t[3];
    Vector3<S> world(const float* x) const {
      Vector3<S> w;
      for (int i = 0; i < 3; ++i)
        w[i] = (S)(t[i] + R[3 * i] * x[0] + R[3 * i + 1] * x[1] + R[3 * i + 2] * x[2]);
      return w;
    }
    Vector3<S> rot(const float* x) const {
      Vector3<S> w;
      for (int i = 0; i < 3; ++i) w[i] = (S)(R[3 * i] * x[0] + R[3 * i + 1] * x[1] + R[3 * i + 2] * x[2]);
      return w;
    }
  };
  uint32_t index_of(const CollisionGeometry<S>* g) {
    auto it = index_.find(g);
    if (it != index_.end()) return it->second;
    const uint32_t k = (uint32_t)shapes_.size();
    detail::encode_shape(g, shapes_, verts_);
    index_[g] = k;
    return k;
  }
  std::vector<fclg_result> run(bool distance, const fclg_request& req) {
    std::vector<fclg_result> r(pairs_.size());
    if (pairs_.empty()) return r;
    fclg_context* ctx = detail::thread_context();
    detail::check(ctx, fclg_set_shapes(ctx, shapes_.data(), (uint32_t)shapes_.size(), verts_.data(), verts_.size() / 4),
                  "fclg_set_shapes");
    const int rc = distance ? fclg_distance(ctx, pairs_.data(), (uint32_t)pairs_.size(), &req, r.data())
                            : fclg_collide(ctx, pairs_.data(), (uint32_t)pairs_.size(), &req, r.data());
    detail::check(ctx, rc, distance ? "fclg_distance" : "fclg_collide");
    return r;
  }
  std::vector<fclg_pair> pairs_;
  std::vector<Frame> frames_;
  std::vector<std::pair<const CollisionGeometry<S>*, const CollisionGeometry<S>*>> geoms_;
  std::vector<fclg_shape> shapes_;
  std::vector<float> verts_;
  std::unordered_map<const CollisionGeometry<S>*, uint32_t> index_;
};

namespace detail {

// Mesh-shape collide with penetration off (MeshShapeIntersect): contacts
// carry the mesh's triangle index (b1 when the mesh is o1, b2 otherwise).
template <typename S, typename TFM, typename TFS>
std::size_t mesh_shape_collide(const CollisionGeometry<S>* mesh, const TFM& tfm, const CollisionGeometry<S>* shape,
                               const TFS& tfs, bool mesh_first, const CollisionRequest<S>& req,
                               CollisionResult<S>& res) {
  using M = BVHModel<OBBRSS<S>>;
  const auto* m = static_cast<const M*>(mesh);
  fclg_context* ctx = thread_context();
  std::vector<fclg_shape> shapes;
  std::vector<float> verts;
  encode_shape(shape, shapes, verts);
  check(ctx, fclg_set_shapes(ctx, shapes.data(), 1, verts.data(), verts.size() / 4), "fclg_set_shapes");
  fclg_pair p{};
  relative_pose(tfm, tfs, p);
  float pose[12];
  for (int i = 0; i < 9; ++i) pose[i] = p.rot[i];
  for (int i = 0; i < 3; ++i) pose[9 + i] = p.trans[i];
  const uint32_t cap = (uint32_t)std::max<std::size_t>(req.maxNumContacts(), 1);
  const uint32_t id = 0;
  uint8_t flag = 0;
  uint32_t count = 0, status = 0;
  std::vector<int32_t> tri((std::size_t)cap, -1);
  // The reference runs a shape-first pair as the mesh-first one (collision-inl.h:90-99): contacts name the
  // mesh as o1 either way.
  (void)mesh_first;
  if (!req.isPenetrationEnabled()) {
    check(ctx, fclg_mesh_shape_collide(ctx, m->device_mesh(ctx), &id, pose, 1, cap, &flag, &count, tri.data(),
                                       &status),
          "fclg_mesh_shape_collide");
    for (uint32_t k = 0; k < count && res.numContacts() < req.maxNumContacts(); ++k)
      res.addContact(Contact<S>(mesh, shape, tri[k], -1));
    return res.numContacts();
  }
  // penetration on: contacts (mesh frame) mapped to the world by the mesh's transform
  std::vector<float> con((std::size_t)cap * 8);
  check(ctx, fclg_mesh_shape_contacts(ctx, m->device_mesh(ctx), &id, pose, 1, cap, &flag, &count, tri.data(),
                                      con.data(), &status),
        "fclg_mesh_shape_contacts");
  for (uint32_t k = 0; k < count && res.numContacts() < req.maxNumContacts(); ++k) {
    const float* q = con.data() + 8 * (std::size_t)k;
    uint32_t st;
    std::memcpy(&st, q + 7, 4);
    if (st & (1u << 8)) continue;  // GJK / EPA found no contact: the reference adds none
    Contact<S> c(mesh, shape, tri[k], -1);
    for (int i = 0; i < 3; ++i) {
      double w = (double)tfm.translation()(i), nw = 0;
      for (int j = 0; j < 3; ++j) {
        w += (double)tfm.linear()(i, j) * (double)q[j];
        nw += (double)tfm.linear()(i, j) * (double)q[3 + j];
      }
      c.pos[i] = (S)w;
      c.normal[i] = (S)nw;
    }
    c.penetration_depth = (S)q[6];
    res.addContact(c);
  }
  return res.numContacts();
}

// Mesh-mesh collide: contacts carry the triangle indices (b1, b2).
template <typename S, typename TF1, typename TF2>
std::size_t mesh_collide(const CollisionGeometry<S>* o1, const TF1& tf1, const CollisionGeometry<S>* o2,
                         const TF2& tf2, const CollisionRequest<S>& req, CollisionResult<S>& res) {
  using M = BVHModel<OBBRSS<S>>;
  const auto* m1 = static_cast<const M*>(o1);
  const auto* m2 = static_cast<const M*>(o2);
  fclg_context* ctx = thread_context();
  fclg_pair p{};
  relative_pose(tf1, tf2, p);
  float pose[12];
  for (int i = 0; i < 9; ++i) pose[i] = p.rot[i];
  for (int i = 0; i < 3; ++i) pose[9 + i] = p.trans[i];
  const uint32_t cap = (uint32_t)std::max<std::size_t>(req.maxNumContacts(), 1);
  uint8_t flag = 0;
  uint32_t count = 0, status = 0;
  std::vector<int32_t> tri(2 * (std::size_t)cap, -1);
  check(ctx,
        fclg_mesh_collide(ctx, m1->device_mesh(ctx), m2->device_mesh(ctx), pose, 1, cap, &flag, &count, tri.data(),
                          &status),
        "fclg_mesh_collide");
  for (uint32_t k = 0; k < count && res.numContacts() < req.maxNumContacts(); ++k)
    res.addContact(Contact<S>(o1, o2, tri[2 * k], tri[2 * k + 1]));
  return res.numContacts();
}

}  // namespace detail

// fcl::collide: shape pairs and BVHModel<OBBRSS> pairs.  Returns the number of
// contacts added to result (at most request.maxNumContacts()).
template <typename S, typename TF1, typename TF2>
std::size_t collide(const CollisionGeometry<S>* o1, const TF1& tf1, const CollisionGeometry<S>* o2, const TF2& tf2,
                    const CollisionRequest<S>& request, CollisionResult<S>& result) {
  if (request.maxNumContacts() == 0) return 0;  // the reference warns and returns 0 (collision-inl.h:73-111)
  const bool m1 = o1->getNodeType() == BV_OBBRSS, m2 = o2->getNodeType() == BV_OBBRSS;
  if (m1 && m2) return detail::mesh_collide(o1, tf1, o2, tf2, request, result);
  if (m1) return detail::mesh_shape_collide(o1, tf1, o2, tf2, true, request, result);
  if (m2) return detail::mesh_shape_collide(o2, tf2, o1, tf1, false, request, result);
  BatchQuery<S> q;
  q.add(o1, tf1, o2, tf2);
  CollisionResult<S> r = q.collide(request).front();
  for (const auto& c : r.getContacts())
    if (result.numContacts() < request.maxNumContacts()) result.addContact(c);
  return r.numContacts();
}

// fcl::translational_ccd (narrowphase/continuous_collision.h:13-19) on shape
// pairs; a BVHModel is not supported here and is reported as the reference
// reports an unsupported pair (a warning, no contact).
template <typename S, typename TF1, typename TF2>
void translational_ccd(const CollisionGeometry<S>* o1, const TF1& tf1,
                       const TranslationalDisplacement<S>& o1_displacement, const CollisionGeometry<S>* o2,
                       const TF2& tf2, const ContinuousCollisionRequest<S>& request,
                       ContinuousCollisionResult<S>& result) {
  if (o1->getNodeType() == BV_OBBRSS || o2->getNodeType() == BV_OBBRSS) {
    std::cerr << "Warning: translational CCD with a BVHModel is not supported\n";
    return;
  }
  if (result.TerminationConditionSatisfied(request.num_max_contacts)) return;
  BatchQuery<S> q;
  q.add(o1, tf1, o2, tf2);
  const auto r = q.translationalCcd({o1_displacement}, request).front();
  for (const auto& c : r.raw_contacts()) result.AddContact(c);
}

// detail::GJKSolver<S>: shapeSignedDistance with the reference's defaults
// (gjk_solver-inl.h:1120-1130); witness points in the world frame.
template <typename S>
class GJKSolver {
 public:
  S gjk_tolerance = S(1e-6);
  template <typename Shape1, typename TF1, typename Shape2, typename TF2>
  bool shapeSignedDistance(const Shape1& s1, const TF1& tf1, const Shape2& s2, const TF2& tf2,
                           S* distance = nullptr, Vector3<S>* p1 = nullptr, Vector3<S>* p2 = nullptr) const {
    BatchQuery<S> q;
    q.add(&s1, tf1, &s2, tf2);
    const auto r = q.signedDistance(gjk_tolerance).front();
    if (distance) *distance = r.ok ? r.distance : S(-1);
    if (r.ok) {
      if (p1) *p1 = r.p1;
      if (p2) *p2 = r.p2;
    }
    return r.ok;
  }
};

}  // namespace fcl
}  // namespace fclg
