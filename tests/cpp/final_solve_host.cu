// Host build of EPA's FP64 final closest-face solve (epa_final_solve in
// mind-fcl_gb300/csrc/device_math.cuh, the function the epa_finalize launch
// and the in-warp solve run) for the CPU tests.  fs_run takes per case the
// face's Minkowski vertices wa, wb, wc, their support points on shape a and
// the fallback support pair (24 floats) and writes p0, p1, depth (7 floats).
#include <cstddef>

#include "device_math.cuh"

extern "C" void fs_run(const float* cases, int n, float* out) {
  for (int i = 0; i < n; ++i) {
    const float* q = cases + 24 * (size_t)i;
    fclg::f3 v[8];
    for (int k = 0; k < 8; ++k) v[k] = fclg::mk3(q[3 * k], q[3 * k + 1], q[3 * k + 2]);
    fclg::f3 p0, p1;
    float depth;
    fclg::epa_final_solve(v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7], p0, p1, depth);
    float* o = out + 7 * (size_t)i;
    o[0] = p0.x;
    o[1] = p0.y;
    o[2] = p0.z;
    o[3] = p1.x;
    o[4] = p1.y;
    o[5] = p1.z;
    o[6] = depth;
  }
}
