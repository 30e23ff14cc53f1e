// Known answers through the fcl-style C++ API (include/fclg_fcl.hpp), from
// the reference's own tests:
//   sphere separation 0.2       test/cvx_collide/test_gjk2_distance.cpp:18-68
//   sphere penetration 0.2      test/cvx_collide/test_epa2_with_gjk2.cpp:21-73
//   box-box flags and depth     test/cvx_collide/test_gjk2.cpp:19-127
// plus a rotated frame (witness points in the world frame), a convex cube,
// the contact cap of fcl::collide and a mesh-mesh collide.
#include <cmath>
#include <cstdio>
#include <memory>
#include <vector>

#include "fclg_fcl.hpp"

using namespace fclg::fcl;
using S = double;

static int failures = 0;
#define CHECK(cond, ...)                        \
  do {                                          \
    if (!(cond)) {                              \
      std::printf("FAIL %s:%d: ", __FILE__, __LINE__); \
      std::printf(__VA_ARGS__);                 \
      std::printf("\n");                        \
      ++failures;                               \
    }                                           \
  } while (0)

static Transform3<S> at(S x, S y, S z) {
  Transform3<S> t;
  t.translation() = Vector3<S>(x, y, z);
  return t;
}

static Transform3<S> rot_z(S ang, S x, S y, S z) {
  Transform3<S> t = at(x, y, z);
  t.linear()(0, 0) = std::cos(ang);
  t.linear()(0, 1) = -std::sin(ang);
  t.linear()(1, 0) = std::sin(ang);
  t.linear()(1, 1) = std::cos(ang);
  return t;
}

int main() {
  GJKSolver<S> solver;
  // spheres of radius 0.5: separated by 0.2, then penetrating by 0.2
  Sphere<S> s1(0.5), s2(0.5);
  S d = 0;
  Vector3<S> p1, p2;
  CHECK(solver.shapeSignedDistance(s1, at(0, 0, 0), s2, at(1.2, 0, 0), &d, &p1, &p2), "sphere distance ok");
  CHECK(std::fabs(d - 0.2) < 1e-4, "sphere separation %.7f", d);
  CHECK(std::fabs(p1[0] - 0.5) < 1e-3 && std::fabs(p2[0] - 0.7) < 1e-3, "witness %.5f %.5f", p1[0], p2[0]);
  CHECK(solver.shapeSignedDistance(s1, at(0, 0, 0), s2, at(0.8, 0, 0), &d), "sphere depth ok");
  CHECK(std::fabs(d + 0.2) < 1e-3, "sphere depth %.7f", d);

  // the same separation in a rotated, translated frame: world-frame witness points
  CHECK(solver.shapeSignedDistance(s1, rot_z(0.7, 1, 2, 3), s2, rot_z(-0.3, 1, 3.2, 3), &d, &p1, &p2), "rot ok");
  CHECK(std::fabs(d - 0.2) < 1e-4, "rotated separation %.7f", d);
  CHECK(std::fabs(p1[1] - 2.5) < 1e-3 && std::fabs(p2[1] - 2.7) < 1e-3, "rotated witness %.5f %.5f", p1[1], p2[1]);

  // unit boxes overlapping by 0.1 along x: boolean, then depth and normal (escape of o2: +x)
  Box<S> b1(1, 1, 1), b2(1, 1, 1);
  CollisionRequest<S> boolean_req;
  CollisionResult<S> res;
  CHECK(collide(&b1, at(0, 0, 0), &b2, at(0.9, 0, 0), boolean_req, res) == 1, "box collide");
  res.clear();
  CHECK(collide(&b1, at(0, 0, 0), &b2, at(1.1, 0, 0), boolean_req, res) == 0, "box separated");
  CollisionRequest<S> pen_req;
  pen_req.useDefaultPenetration();
  res.clear();
  collide(&b1, at(0, 0, 0), &b2, at(0.9, 0.05, 0), pen_req, res);
  CHECK(res.isCollision(), "box contact");
  if (res.isCollision()) {
    const auto& c = res.getContact(0);
    CHECK(std::fabs(c.penetration_depth - 0.1) < 1e-4, "box depth %.7f", c.penetration_depth);
    CHECK(c.normal[0] > 0.999, "box normal %.4f %.4f %.4f", c.normal[0], c.normal[1], c.normal[2]);
    CHECK(c.o1 == &b1 && c.o2 == &b2, "contact objects");
  }
  CollisionRequest<S> zero_req(0);
  res.clear();
  CHECK(collide(&b1, at(0, 0, 0), &b2, at(0.5, 0, 0), zero_req, res) == 0, "no contacts requested");

  // MPR penetration modes: b2 sits 0.2 deep on top of b1.  Directed along +z
  // gives 0.2; incremental from a tilted hint settles on +z with 0.2.
  CollisionRequest<S> dir_req;
  dir_req.useDirectedPenetration(Vector3<S>(0, 0, 1));
  res.clear();
  collide(&b1, at(0, 0, 0), &b2, at(0.05, 0.02, 0.8), dir_req, res);
  CHECK(res.isCollision(), "directed contact");
  if (res.isCollision()) {
    const auto& c = res.getContact(0);
    CHECK(std::fabs(c.penetration_depth - 0.2) < 1e-4, "directed depth %.7f", c.penetration_depth);
    CHECK(c.normal[2] > 0.9999, "directed normal %.4f %.4f %.4f", c.normal[0], c.normal[1], c.normal[2]);
  }
  CollisionRequest<S> inc_req;
  const S h = S(1) / std::sqrt(S(1.04));
  inc_req.useIncrementalMinimumDistancePenetration(Vector3<S>(S(0.2) * h, 0, h));
  res.clear();
  collide(&b1, at(0, 0, 0), &b2, at(0.05, 0.02, 0.8), inc_req, res);
  CHECK(res.isCollision(), "incremental contact");
  if (res.isCollision()) {
    const auto& c = res.getContact(0);
    CHECK(std::fabs(c.penetration_depth - 0.2) < 1e-4, "incremental depth %.7f", c.penetration_depth);
    CHECK(c.normal[2] > 0.999, "incremental normal %.4f %.4f %.4f", c.normal[0], c.normal[1], c.normal[2]);
  }

  // convex cube (8 vertices) against a sphere: distance 0.3
  auto verts = std::make_shared<std::vector<Vector3<S>>>();
  for (int i = 0; i < 8; ++i) verts->push_back(Vector3<S>((i & 1) ? 0.5 : -0.5, (i & 2) ? 0.5 : -0.5, (i & 4) ? 0.5 : -0.5));
  auto faces = std::make_shared<std::vector<int>>();
  Convex<S> cube(verts, 6, faces);
  CHECK(solver.shapeSignedDistance(cube, at(0, 0, 0), s2, at(0, 0, 1.3), &d), "convex ok");
  CHECK(std::fabs(d - 0.3) < 1e-4, "convex-sphere %.7f", d);

  // batch: 1000 sphere pairs at growing distance, one call
  BatchQuery<S> batch;
  for (int i = 0; i < 1000; ++i) batch.add(&s1, at(0, 0, 0), &s2, at(0.5 + 0.001 * i, 0, 0));
  const auto out = batch.signedDistance();
  int bad = 0;
  for (int i = 0; i < 1000; ++i) {
    const S want = 0.5 + 0.001 * i - 1.0;
    if (!out[i].ok || std::fabs(out[i].distance - want) > 2e-3) ++bad;
  }
  CHECK(bad == 0, "batch sphere pairs off: %d", bad);

  // meshes: two octahedra, overlapping and apart
  std::vector<Vector3<S>> pts = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
  std::vector<Triangle> tris = {{0, 2, 4}, {2, 1, 4}, {1, 3, 4}, {3, 0, 4}, {2, 0, 5}, {1, 2, 5}, {3, 1, 5}, {0, 3, 5}};
  BVHModel<OBBRSS<S>> m1, m2;
  m1.beginModel();
  m1.addSubModel(pts, tris);
  m1.endModel();
  m2.beginModel();
  m2.addSubModel(pts, tris);
  m2.endModel();
  CollisionRequest<S> mesh_req(4);
  res.clear();
  CHECK(collide(&m1, at(0, 0, 0), &m2, at(1.5, 0, 0), mesh_req, res) > 0, "mesh overlap");
  for (const auto& c : res.getContacts()) CHECK(c.b1 >= 0 && c.b1 < 8 && c.b2 >= 0 && c.b2 < 8, "triangle ids");
  res.clear();
  CHECK(collide(&m1, at(0, 0, 0), &m2, at(2.5, 0, 0), mesh_req, res) == 0, "mesh apart");

  // mesh-shape (MeshShapeIntersect): a sphere and a box crossing the mesh's
  // surface collide, a sphere outside it does not
  Sphere<S> ball(0.3);
  CollisionRequest<S> ms_req(4);
  res.clear();
  CHECK(collide(&m1, at(0, 0, 0), &ball, at(1.1, 0, 0), ms_req, res) > 0, "mesh-sphere overlap");
  for (const auto& c : res.getContacts()) CHECK(c.o1 == &m1 && c.b1 >= 0 && c.b1 < 8, "mesh-sphere triangle ids");
  res.clear();
  CHECK(collide(&m1, at(0, 0, 0), &ball, at(2.0, 0, 0), ms_req, res) == 0, "mesh-sphere apart");
  res.clear();
  CHECK(collide(&b1, at(0.9, 0, 0), &m1, at(0, 0, 0), ms_req, res) > 0, "box-mesh overlap");
  // a shape-first pair runs as the mesh-first one: the mesh is o1 (collision-inl.h:90-99)
  for (const auto& c : res.getContacts()) CHECK(c.o1 == &m1 && c.b1 >= 0 && c.b1 < 8, "box-mesh triangle ids");

  // with penetration: a sphere of radius 0.3 centred 1.1 along +x from the octahedron's centre dips 0.2
  // into its vertex region; contacts carry a depth and a unit normal
  CollisionRequest<S> ms_pen(4);
  ms_pen.useDefaultPenetration();
  res.clear();
  CHECK(collide(&m1, at(0, 0, 0), &ball, at(1.1, 0, 0), ms_pen, res) > 0, "mesh-sphere contact");
  for (const auto& c : res.getContacts()) {
    const S nn = std::sqrt(c.normal[0] * c.normal[0] + c.normal[1] * c.normal[1] + c.normal[2] * c.normal[2]);
    CHECK(std::fabs(nn - 1) < 1e-4 && c.penetration_depth < 0 && c.penetration_depth > -0.3,
          "mesh-sphere contact depth %.5f normal %.5f", (double)c.penetration_depth, (double)nn);
  }
  res.clear();
  CHECK(collide(&m1, at(0, 0, 0), &b1, at(0.9, 0, 0), ms_pen, res) > 0, "mesh-box contact");
  for (const auto& c : res.getContacts())
    CHECK(c.penetration_depth > 0 && c.penetration_depth < 1.0, "mesh-box depth %.5f", (double)c.penetration_depth);

  // translational CCD (test/ccd/test_shape_pair_interface.cpp): a sphere of
  // radius 0.1 moving 1 along +x towards a sphere of radius 0.125 at x = 0.6
  // hits; at x = 1.3 it stops short; moving along -x it never reaches it.  The
  // sampled time puts the spheres in touch; two unit cubes 3 apart meet
  // within the box interval [0.5, 1] of a motion of 4 along +x.
  {
    Sphere<S> a(0.1), b(0.125);
    TranslationalDisplacement<S> mv;
    mv.unit_axis_in_shape1 = Vector3<S>(1, 0, 0);
    mv.scalar_displacement = 1.0;
    ContinuousCollisionRequest<S> creq;
    creq.request_type = TimeOfCollisionRequestType::kOneTocSample;
    ContinuousCollisionResult<S> cres;
    translational_ccd<S>(&a, at(0, 0, 0), mv, &b, at(0.6, 0, 0), creq, cres);
    CHECK(cres.num_contacts() == 1, "ccd sphere hit");
    if (cres.num_contacts() == 1) {
      const S t = cres.raw_contacts()[0].toc.lower_bound;
      CHECK(t >= 0 && t <= 1 && std::fabs(0.6 - t) <= 0.225 + 1e-5, "ccd sphere toc %.6f", t);
      CHECK(cres.raw_contacts()[0].o1 == &a && cres.raw_contacts()[0].o2 == &b, "ccd contact objects");
    }
    ContinuousCollisionResult<S> far;
    translational_ccd<S>(&a, at(0, 0, 0), mv, &b, at(1.3, 0, 0), creq, far);
    CHECK(far.num_contacts() == 0, "ccd sphere stops short");
    mv.unit_axis_in_shape1 = Vector3<S>(-1, 0, 0);
    ContinuousCollisionResult<S> back;
    translational_ccd<S>(&a, at(0, 0, 0), mv, &b, at(0.6, 0, 0), creq, back);
    CHECK(back.num_contacts() == 0, "ccd sphere moving away");
    Box<S> c1(1, 1, 1), c2(1, 1, 1);
    mv.unit_axis_in_shape1 = Vector3<S>(1, 0, 0);
    mv.scalar_displacement = 4.0;
    ContinuousCollisionRequest<S> breq;
    ContinuousCollisionResult<S> bres;
    translational_ccd<S>(&c1, at(0, 0, 0), mv, &c2, at(3, 0, 0), breq, bres);
    CHECK(bres.num_contacts() == 1, "ccd boxes hit");
    if (bres.num_contacts() == 1)
      CHECK(std::fabs(bres.raw_contacts()[0].toc.lower_bound - 0.5) < 1e-6 &&
                std::fabs(bres.raw_contacts()[0].toc.upper_bound - 1.0) < 1e-6,
            "ccd box interval [%.6f, %.6f]", bres.raw_contacts()[0].toc.lower_bound,
            bres.raw_contacts()[0].toc.upper_bound);
  }

  if (failures == 0) std::printf("fcl_compat_test: all passed\n");
  return failures == 0 ? 0 : 1;
}
