// Host build of the FP64 GJK (mind-fcl_gb300/csrc/gjk64.cuh) for the CPU
// tests: the same functions the FP64 kernel (fp64_pass.cu) runs, compiled with
// -ffp-contract=off so each operation rounds once as on the device.  g64_run
// mirrors gjk64_pass pair for pair and writes fclg_result64 records.
#include <cstdint>

struct float4 {
  float x, y, z, w;
};
namespace fclg {
// the shape and GJK status codes of device_math.cuh
enum : int32_t { kBox = 0, kSphere = 1, kCapsule = 3, kCylinder = 5, kConvex = 100 };
enum : int32_t { kGjkIntersect = 0, kGjkSeparated = 1, kGjkNoProgress = 2, kGjkIterLimit = 3, kGjkFailed = 4 };
struct ShapeDev {
  int32_t type;
  uint32_t vofs, nv;
  float p0, p1, p2;
};
}  // namespace fclg

#define FCLG64_HOST
#include "gjk64.cuh"

namespace {
struct ShapeRec {  // fclg_shape
  int32_t type;
  uint32_t vert_offset, vert_count, reserved;
  float param[4];
};
struct PairRec {  // fclg_pair
  uint32_t a, b;
  float rot[9], trans[3];
  uint32_t flags, pair_class;
};
struct Result64 {  // fclg_result64
  double distance, p_a[3], p_b[3];
  int32_t status;
  uint16_t iterations;
  uint8_t collide, ok;
};
static_assert(sizeof(Result64) == 64, "fclg_result64");

fclg::ShapeDev decode(const ShapeRec& r) {  // device_math.cuh load_shape
  fclg::ShapeDev s;
  s.type = r.type;
  s.vofs = r.vert_offset;
  s.nv = r.vert_count;
  if (s.type == fclg::kBox) {
    s.p0 = 0.5f * r.param[0];
    s.p1 = 0.5f * r.param[1];
    s.p2 = 0.5f * r.param[2];
  } else {
    s.p0 = r.param[0];
    s.p1 = 0.5f * r.param[1];
    s.p2 = 0.f;
  }
  return s;
}
}  // namespace

extern "C" void g64_run(const void* shapes, uint32_t n_shapes, const void* verts, const void* pairs, uint32_t n,
                        double tol, int max_iter, void* out) {
  using namespace fclg;
  const ShapeRec* sh = static_cast<const ShapeRec*>(shapes);
  const PairRec* pr = static_cast<const PairRec*>(pairs);
  Result64* res = static_cast<Result64*>(out);
  for (uint32_t i = 0; i < n; ++i) {
    Result64 r{};
    r.distance = -1.;
    r.status = kGjkFailed;
    if (pr[i].a < n_shapes && pr[i].b < n_shapes) {
      f64::MinkowskiSupport64 sup;
      sup.A = decode(sh[pr[i].a]);
      sup.B = decode(sh[pr[i].b]);
      for (int k = 0; k < 9; ++k) sup.pose.r[k] = pr[i].rot[k];
      sup.pose.t = f64::v3{pr[i].trans[0], pr[i].trans[1], pr[i].trans[2]};
      sup.verts = static_cast<const float4*>(verts);
      f64::Simplex s;
      const f64::GjkOut o = f64::gjk_evaluate(sup, f64::v3{-1., 0., 0.}, tol, max_iter, true, s);
      r.status = o.status;
      r.iterations = (uint16_t)(o.iterations > 0xFFFF ? 0xFFFF : o.iterations);
      r.collide = o.status == kGjkIntersect;
      if (o.status == kGjkSeparated && o.point_valid) {
        r.ok = 1;
        r.distance = f64::nrm(o.p0 - o.p1);
        r.p_a[0] = o.p0.x; r.p_a[1] = o.p0.y; r.p_a[2] = o.p0.z;
        r.p_b[0] = o.p1.x; r.p_b[1] = o.p1.y; r.p_b[2] = o.p1.z;
      }
    }
    res[i] = r;
  }
}
