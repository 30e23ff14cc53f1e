// The plain method in FP64 on the GPU: GJKSolver<double>::shapeDistance
// (narrowphase/detail/gjk_solver-inl.h:760-798) per pair, one thread per pair
// (gjk64.cuh).  It is the baseline the FP32 kernels are a change from: the
// same batch and pair records, FP64 arithmetic throughout, FP64 results.
#include "gjk64.cuh"
#include "kernels.h"

namespace fclg {

namespace {

__global__ void __launch_bounds__(128) gjk64_pass(BatchArgs b, double tol, int max_iter, double* __restrict__ out) {
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t pid = blockIdx.x * blockDim.x + threadIdx.x; pid < b.n_pairs; pid += stride) {
    const PairDev pr = load_pair(b.pairs, pid);
    double* o = out + 8 * (size_t)pid;  // fclg_result64: 8 doubles
    int32_t status = kGjkFailed;
    uint32_t iters = 0;
    bool collide = false, ok = false;
    double dist = -1.0;
    f64::v3 p0{0., 0., 0.}, p1{0., 0., 0.};
    if (pr.a < b.n_shapes && pr.b < b.n_shapes) {
      f64::MinkowskiSupport64 sup;
      sup.A = load_shape(b.shapes, pr.a);
      sup.B = load_shape(b.shapes, pr.b);
      for (int k = 0; k < 9; ++k) sup.pose.r[k] = pr.pose.r[k];
      sup.pose.t = f64::v3{pr.pose.t.x, pr.pose.t.y, pr.pose.t.z};
      sup.verts = b.verts;
      f64::Simplex s;
      // GJKSolver's default guess (1, 0, 0), gjk_solver-inl.h:1129; Evaluate(-guess)
      const f64::GjkOut r = f64::gjk_evaluate(sup, f64::v3{-1., 0., 0.}, tol, max_iter, true, s);
      status = r.status;
      iters = (uint32_t)r.iterations;
      collide = r.status == kGjkIntersect;
      if (r.status == kGjkSeparated && r.point_valid) {
        // shapeDistance: separated -> the distance between the witness points
        ok = true;
        p0 = r.p0;
        p1 = r.p1;
        dist = f64::nrm(p0 - p1);
      }
    }
    o[0] = dist;
    o[1] = p0.x;
    o[2] = p0.y;
    o[3] = p0.z;
    o[4] = p1.x;
    o[5] = p1.y;
    o[6] = p1.z;
    const uint32_t w0 = (uint32_t)status;
    const uint32_t w1 = (iters > 0xFFFFu ? 0xFFFFu : iters) | ((collide ? 1u : 0u) << 16) | ((ok ? 1u : 0u) << 24);
    o[7] = __hiloint2double((int)w1, (int)w0);
  }
}

}  // namespace

cudaError_t launch_gjk64(const BatchArgs& b, double tol, int max_iter, double* out, int blocks, cudaStream_t st) {
  if (b.n_pairs == 0) return cudaSuccess;
  const uint32_t need = (b.n_pairs + 127) / 128;
  gjk64_pass<<<(int)(need < (uint32_t)blocks ? need : (uint32_t)blocks), 128, 0, st>>>(b, tol, max_iter, out);
  return cudaGetLastError();
}

}  // namespace fclg
