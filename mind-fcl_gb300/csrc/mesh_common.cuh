// OBB tree nodes and the FP32 box-overlap test shared by the mesh kernels
// (mesh_query.cu, mesh_shape.cu).
#pragma once
#include "device_math.cuh"

namespace fclg {

struct Node {
  float a[9];  // row-major, columns are the axes
  f3 c;
  f3 e;
  int32_t child;
};

__device__ __forceinline__ Node load_node(const float4* __restrict__ nodes, uint32_t i) {
  const float4 q0 = __ldg(nodes + 4 * (size_t)i);
  const float4 q1 = __ldg(nodes + 4 * (size_t)i + 1);
  const float4 q2 = __ldg(nodes + 4 * (size_t)i + 2);
  const float4 q3 = __ldg(nodes + 4 * (size_t)i + 3);
  Node n;
  n.a[0] = q0.x; n.a[1] = q0.y; n.a[2] = q0.z; n.a[3] = q0.w;
  n.a[4] = q1.x; n.a[5] = q1.y; n.a[6] = q1.z; n.a[7] = q1.w;
  n.a[8] = q2.x;
  n.c = mk3(q2.y, q2.z, q2.w);
  n.e = mk3(q3.x, q3.y, q3.z);
  n.child = __float_as_int(q3.w);
  return n;
}

// FP32 OBB overlap, conservative: |R| gets 1e-5 (the reference 1e-6) and
// every comparison an absolute slack.
__device__ __forceinline__ bool obb_overlap(const Pose& P, const Node& A, const Node& B) {
  constexpr float reps = 1e-5f;
  constexpr float slack = 4e-6f;
  float R0b2[9];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c)
      R0b2[3 * r + c] = fmaf(P.r[3 * r + 2], B.a[6 + c], fmaf(P.r[3 * r + 1], B.a[3 + c], P.r[3 * r] * B.a[c]));
  float R[9], F[9];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      R[3 * r + c] = fmaf(A.a[6 + r], R0b2[6 + c], fmaf(A.a[3 + r], R0b2[3 + c], A.a[r] * R0b2[c]));
      F[3 * r + c] = fabsf(R[3 * r + c]) + reps;
    }
  const f3 tt = P.rot(B.c) + P.t - A.c;
  const float T0 = fmaf(tt.z, A.a[6], fmaf(tt.y, A.a[3], tt.x * A.a[0]));
  const float T1 = fmaf(tt.z, A.a[7], fmaf(tt.y, A.a[4], tt.x * A.a[1]));
  const float T2 = fmaf(tt.z, A.a[8], fmaf(tt.y, A.a[5], tt.x * A.a[2]));
  const float a0 = A.e.x, a1 = A.e.y, a2 = A.e.z, b0 = B.e.x, b1 = B.e.y, b2 = B.e.z;
  if (fabsf(T0) > a0 + F[0] * b0 + F[1] * b1 + F[2] * b2 + slack) return false;
  if (fabsf(T1) > a1 + F[3] * b0 + F[4] * b1 + F[5] * b2 + slack) return false;
  if (fabsf(T2) > a2 + F[6] * b0 + F[7] * b1 + F[8] * b2 + slack) return false;
  if (fabsf(R[0] * T0 + R[3] * T1 + R[6] * T2) > b0 + F[0] * a0 + F[3] * a1 + F[6] * a2 + slack) return false;
  if (fabsf(R[1] * T0 + R[4] * T1 + R[7] * T2) > b1 + F[1] * a0 + F[4] * a1 + F[7] * a2 + slack) return false;
  if (fabsf(R[2] * T0 + R[5] * T1 + R[8] * T2) > b2 + F[2] * a0 + F[5] * a1 + F[8] * a2 + slack) return false;
  if (fabsf(T2 * R[3] - T1 * R[6]) > a1 * F[6] + a2 * F[3] + b1 * F[2] + b2 * F[1] + slack) return false;
  if (fabsf(T2 * R[4] - T1 * R[7]) > a1 * F[7] + a2 * F[4] + b0 * F[2] + b2 * F[0] + slack) return false;
  if (fabsf(T2 * R[5] - T1 * R[8]) > a1 * F[8] + a2 * F[5] + b0 * F[1] + b1 * F[0] + slack) return false;
  if (fabsf(T0 * R[6] - T2 * R[0]) > a0 * F[6] + a2 * F[0] + b1 * F[5] + b2 * F[4] + slack) return false;
  if (fabsf(T0 * R[7] - T2 * R[1]) > a0 * F[7] + a2 * F[1] + b0 * F[5] + b2 * F[3] + slack) return false;
  if (fabsf(T0 * R[8] - T2 * R[2]) > a0 * F[8] + a2 * F[2] + b0 * F[4] + b1 * F[3] + slack) return false;
  if (fabsf(T1 * R[0] - T0 * R[3]) > a0 * F[3] + a1 * F[0] + b1 * F[8] + b2 * F[7] + slack) return false;
  if (fabsf(T1 * R[1] - T0 * R[4]) > a0 * F[4] + a1 * F[1] + b0 * F[8] + b2 * F[6] + slack) return false;
  if (fabsf(T1 * R[2] - T0 * R[5]) > a0 * F[5] + a1 * F[2] + b0 * F[7] + b1 * F[6] + slack) return false;
  return true;
}

// Ordered traversal (both mesh kernels).  A pending node (pair) carries its
// path key: the descent choices from the root, one bit per step (0 = the
// child the reference visits first), left-aligned above a sentinel bit, so
// that two keys compare as unsigned integers as their places in the
// reference's depth-first visiting order.  Paths hold at most 62 steps.
constexpr unsigned long long kRootKey = 1ull << 63;
constexpr unsigned long long kNoKey = ~0ull;

__device__ __forceinline__ unsigned long long child_key(unsigned long long k, unsigned later) {
  const unsigned long long low = k & (~k + 1ull);  // sentinel
  return (k & ~low) | (later ? low : 0ull) | (low >> 1);
}

__device__ __forceinline__ int pow2_at_least(int n) {
  int p = 2;
  while (p < n) p <<= 1;
  return p;
}

// Sorts the first n2 (a power of two, n2 >= 2) buffer entries by key,
// ascending: a bitonic network, the warp's lanes taking the compare-exchange
// pairs of each step.
__device__ __forceinline__ void warp_sort_keys(unsigned long long* key, int2* val, int n2, unsigned lane) {
  for (int k = 2; k <= n2; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = (int)lane; i < n2; i += 32) {
        const int l = i ^ j;
        if (l > i) {
          const unsigned long long ki = key[i], kl = key[l];
          const bool up = (i & k) == 0;
          if (up ? (ki > kl) : (ki < kl)) {
            key[i] = kl;
            key[l] = ki;
            const int2 t = val[i];
            val[i] = val[l];
            val[l] = t;
          }
        }
      }
      __syncwarp();
    }
  }
}

// Contacts kept in key order: entries [0, found) of (key, value) with
// max_contacts + 32 slots.  After a round appended its hits, keep() sorts and
// cuts to max_contacts once the buffer holds that many, and returns the key of
// the last kept contact (kNoKey while fewer).
__device__ __forceinline__ unsigned long long keep_first(unsigned long long* key, int2* val, int& found, int cap,
                                                         unsigned lane, unsigned long long last) {
  if (found < cap) return last;
  const int n2 = pow2_at_least(found);
  for (int i = found + (int)lane; i < n2; i += 32) key[i] = kNoKey;
  __syncwarp();
  warp_sort_keys(key, val, n2, lane);
  found = cap;
  const unsigned long long l = key[cap - 1];
  __syncwarp();
  return l;
}

// Final order of a buffer that never filled (found < max_contacts).
__device__ __forceinline__ void sort_found(unsigned long long* key, int2* val, int found, int cap, unsigned lane) {
  if (found <= 0 || found >= cap) return;
  const int n2 = pow2_at_least(found);
  for (int i = found + (int)lane; i < n2; i += 32) key[i] = kNoKey;
  __syncwarp();
  warp_sort_keys(key, val, n2, lane);
}

__device__ __forceinline__ f3 ldv(const float4* __restrict__ tris, uint32_t t, int k) {
  const float4 q = __ldg(tris + 3 * (size_t)t + k);
  return mk3(q.x, q.y, q.z);
}

}  // namespace fclg
