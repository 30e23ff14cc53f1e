// Learned warm start: a small MLP that predicts, from the relative pose of a
// pair and a learned embedding of its shape-pair class, the unit direction
// GJK starts its search from (GJKSolver::gjk_guess, gjk_solver-inl.h:1129;
// GJK::Evaluate(shape, -guess), gjk_solver-inl.h:86-90).  The reference has no
// learned component; this file is the whole of it.
//
// Model (all sizes fixed):
//   x  = [R (9, row-major), t (3), E[pair_class] (16), 0 (4)]         32
//   h1 = gelu(W1 x + b1)   h2 = gelu(W2 h1 + b2)   h3 = gelu(W3 h2 + b3)   256 each
//   (gelu in its tanh form, see below)
//   y  = W4 h3 + b4 (rows 3..7 of W4 are zero padding)   guess = y / |y|
// Storage: FP32 master parameters (flat, layout below) and BF16 copies of the
// weight matrices and the embedding table for the tensor-core products; every
// product accumulates in FP32 (mma.sync m16n8k16 BF16 -> FP32).  Activations
// between layers are BF16, pre-activations FP32.
//
// Training (Adam on the FP32 master copy) minimises the mean of
// 1 - <y / |y|, u> over pairs, u the unit direction plain-initialised GJK ends
// at.  Forward and backward run as tiled BF16 GEMMs with fused epilogues
// (bias + GELU, GELU derivative, embedding scatter); inference runs as one
// fused kernel per 128-pair tile with each layer's weights staged in shared
// memory.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "fclg.h"
#include "warmstart.h"

namespace fclg {
namespace wsm {

constexpr int kIn = 32;
constexpr int kH = 256;
constexpr int kOut = 8;
constexpr int kEmb = 16;
constexpr int kPoseCols = 12;

// FP32 master parameter layout (floats)
constexpr size_t oW1 = 0, oB1 = oW1 + (size_t)kH * kIn;
constexpr size_t oW2 = oB1 + kH, oB2 = oW2 + (size_t)kH * kH;
constexpr size_t oW3 = oB2 + kH, oB3 = oW3 + (size_t)kH * kH;
constexpr size_t oW4 = oB3 + kH, oB4 = oW4 + (size_t)kOut * kH;
constexpr size_t oE = oB4 + kOut;
// BF16 copy layout (elements)
constexpr size_t qW1 = 0, qW2 = qW1 + (size_t)kH * kIn, qW3 = qW2 + (size_t)kH * kH, qW4 = qW3 + (size_t)kH * kH;
constexpr size_t qE = qW4 + (size_t)kOut * kH;

typedef __nv_bfloat16 bf16;

__host__ __device__ inline size_t param_count(uint32_t n_classes) { return oE + (size_t)kEmb * n_classes; }

// BF16 slot of master parameter i, or -1 for a bias.
__device__ __forceinline__ long long bf16_slot(size_t i) {
  if (i < oB1) return (long long)(qW1 + i);
  if (i < oW2) return -1;
  if (i < oB2) return (long long)(qW2 + (i - oW2));
  if (i < oW3) return -1;
  if (i < oB3) return (long long)(qW3 + (i - oW3));
  if (i < oW4) return -1;
  if (i < oB4) return (long long)(qW4 + (i - oW4));
  if (i < oE) return -1;
  return (long long)(qE + (i - oE));
}

// GELU in its tanh form (Hendrycks & Gimpel, 2016):
//   gelu(x) = x / 2 (1 + tanh(c (x + a x^3))),  c = sqrt(2 / pi), a = 0.044715.
// Training uses tanhf; inference the hardware tanh.approx.f32 (one MUFU op,
// relative error about 2^-11, below the BF16 resolution of the activations).
constexpr float kGeluC = 0.79788456080286536f;
constexpr float kGeluA = 0.044715f;

__device__ __forceinline__ float tanh_fast(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float gelu(float x) {
  return 0.5f * x * (1.f + tanhf(kGeluC * fmaf(kGeluA * x, x * x, x)));
}
// The same function as h + h tanh(x (c + c a x^2)), h = x / 2: five FP32
// operations and the MUFU tanh.
__device__ __forceinline__ float gelu_fast(float x) {
  const float h = 0.5f * x;
  return fmaf(h, tanh_fast(x * fmaf(kGeluC * kGeluA, x * x, kGeluC)), h);
}
__device__ __forceinline__ float gelu_grad(float x) {
  const float t = tanhf(kGeluC * fmaf(kGeluA * x, x * x, x));
  return 0.5f * (1.f + t) + 0.5f * x * (1.f - t * t) * kGeluC * fmaf(3.f * kGeluA, x * x, 1.f);
}

__device__ __forceinline__ void mma_bf16(float* c, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ uint32_t ld_pair(const bf16* p) { return *reinterpret_cast<const uint32_t*>(p); }

// Feature value of column c for a pair record q (16 words) and embedding row e.
__device__ __forceinline__ float feature(const float* q, const bf16* e, int c) {
  if (c < 9) return q[2 + c];
  if (c < kPoseCols) return q[11 + (c - 9)];
  if (c < kPoseCols + kEmb) return __bfloat162float(e[c - kPoseCols]);
  return 0.f;
}

}  // namespace wsm
}  // namespace fclg

#include "warmstart_tc.cuh"

namespace fclg {
namespace wsm {

// ---------------------------------------------------------------- training --

// X0[m][0..31] for the pairs order[m] (or m), m < M (rows past n are zero).
__global__ void features_kernel(const float4* __restrict__ pairs, const uint32_t* __restrict__ order, uint32_t n,
                                uint32_t M, const bf16* __restrict__ emb, uint32_t n_classes, bf16* __restrict__ X0,
                                uint32_t* __restrict__ cls_out) {
  const uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= M) return;
  bf16* row = X0 + (size_t)m * kIn;
  if (m >= n) {
    for (int c = 0; c < kIn; ++c) row[c] = __float2bfloat16(0.f);
    cls_out[m] = 0xFFFFFFFFu;
    return;
  }
  const uint32_t pid = order ? order[m] : m;
  float q[16];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const float4 v = __ldg(pairs + 4 * (size_t)pid + j);
    q[4 * j] = v.x;
    q[4 * j + 1] = v.y;
    q[4 * j + 2] = v.z;
    q[4 * j + 3] = v.w;
  }
  uint32_t cls = __float_as_uint(q[15]);
  if (cls >= n_classes) cls = 0;
  cls_out[m] = cls;
  const bf16* e = emb + (size_t)cls * kEmb;
  for (int c = 0; c < kIn; ++c) row[c] = __float2bfloat16(feature(q, e, c));
}

struct GemmArgs {
  const bf16* A;
  long long sam, sak;  // A(m, k) = A[m * sam + k * sak]
  const bf16* B;
  long long sbk, sbn;  // B(k, n) = B[k * sbk + n * sbn]
  int M, N, K;
  int k_chunk;         // K range per blockIdx.z
};

// Epilogue: Z = acc + b (optional), A = bf16(gelu(Z) or Z) (optional), Y = fp32 (optional).
struct EpiForward {
  const float* bias;
  float* Z;
  bf16* Aout;
  float* Y;
  int ld;
  bool gelu_on;
  __device__ void operator()(int m, int n, float v) const {
    v += bias[n];
    if (Z) Z[(size_t)m * ld + n] = v;
    const float a = gelu_on ? gelu(v) : v;
    if (Aout) Aout[(size_t)m * ld + n] = __float2bfloat16(a);
    if (Y) Y[(size_t)m * ld + n] = a;
  }
};

// Epilogue of dX = dZ W: times gelu'(Zprev), stored BF16.
struct EpiBackGelu {
  const float* Zprev;
  bf16* dZprev;
  int ld;
  __device__ void operator()(int m, int n, float v) const {
    dZprev[(size_t)m * ld + n] = __float2bfloat16(v * gelu_grad(Zprev[(size_t)m * ld + n]));
  }
};

// Epilogue of dX0 = dZ1 W1: embedding columns scatter into the table gradient.
struct EpiEmbed {
  const uint32_t* cls;
  float* dE;
  __device__ void operator()(int m, int n, float v) const {
    if (n < kPoseCols || n >= kPoseCols + kEmb) return;
    const uint32_t c = cls[m];
    if (c == 0xFFFFFFFFu) return;
    atomicAdd(dE + (size_t)c * kEmb + (n - kPoseCols), v);
  }
};

// Epilogue of dW = dZ^T X (split over K): accumulate into the gradient.
struct EpiAccum {
  float* G;
  int ld;
  __device__ void operator()(int m, int n, float v) const { atomicAdd(G + (size_t)m * ld + n, v); }
};

// C(M x N) = A(M x K) B(K x N), BF16 inputs, FP32 accumulation; 64 x 64 CTA
// tiles of four warps (32 x 32 each), K in steps of 32 staged in shared
// memory; K split over gridDim.z in chunks of k_chunk.
template <class Epi>
__global__ void __launch_bounds__(128) gemm_kernel(GemmArgs g, Epi epi) {
  __shared__ __align__(16) bf16 As[64][40];
  __shared__ __align__(16) bf16 Bs[64][40];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int wm = warp >> 1, wn = warp & 1;
  const int gid = lane >> 2, tig = lane & 3;
  const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
  const int kb = blockIdx.z * g.k_chunk;
  const int ke = min(g.K, kb + g.k_chunk);
  const bf16 zero = __float2bfloat16(0.f);
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;
  for (int k0 = kb; k0 < ke; k0 += 32) {
    for (int idx = tid; idx < 64 * 32; idx += 128) {
      int r, c;
      if (g.sak == 1) { r = idx >> 5; c = idx & 31; }
      else { r = idx & 63; c = idx >> 6; }
      const int m = m0 + r, k = k0 + c;
      As[r][c] = (m < g.M && k < ke) ? g.A[(long long)m * g.sam + (long long)k * g.sak] : zero;
    }
    for (int idx = tid; idx < 64 * 32; idx += 128) {
      int r, c;
      if (g.sbk == 1) { r = idx >> 5; c = idx & 31; }
      else { r = idx & 63; c = idx >> 6; }
      const int n = n0 + r, k = k0 + c;
      Bs[r][c] = (n < g.N && k < ke) ? g.B[(long long)k * g.sbk + (long long)n * g.sbn] : zero;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 32; kk += 16) {
      uint32_t af[2][4], bfr[4][2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int r = wm * 32 + i * 16 + gid;
        af[i][0] = ld_pair(&As[r][kk + 2 * tig]);
        af[i][1] = ld_pair(&As[r + 8][kk + 2 * tig]);
        af[i][2] = ld_pair(&As[r][kk + 2 * tig + 8]);
        af[i][3] = ld_pair(&As[r + 8][kk + 2 * tig + 8]);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int n = wn * 32 + j * 8 + gid;
        bfr[j][0] = ld_pair(&Bs[n][kk + 2 * tig]);
        bfr[j][1] = ld_pair(&Bs[n][kk + 2 * tig + 8]);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], af[i], bfr[j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int r0 = m0 + wm * 32 + i * 16 + gid;
      const int c0 = n0 + wn * 32 + j * 8 + 2 * tig;
#pragma unroll
      for (int h = 0; h < 4; ++h) {
        const int m = r0 + (h >> 1) * 8, n = c0 + (h & 1);
        if (m < g.M && n < g.N) epi(m, n, acc[i][j][h]);
      }
    }
}

// Cosine loss and its gradient with respect to y (rows m < n_valid).
__global__ void loss_kernel(const float* __restrict__ Y, const float* __restrict__ labels,
                            const uint32_t* __restrict__ order, uint32_t n_valid, uint32_t M, float inv_n,
                            bf16* __restrict__ dY, float* __restrict__ loss_sum) {
  const uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.f;
  if (m < M) {
    float g[kOut] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (m < n_valid) {
      const uint32_t pid = order ? order[m] : m;
      const float y0 = Y[(size_t)m * kOut], y1 = Y[(size_t)m * kOut + 1], y2 = Y[(size_t)m * kOut + 2];
      const float u0 = labels[3 * (size_t)pid], u1 = labels[3 * (size_t)pid + 1], u2 = labels[3 * (size_t)pid + 2];
      const float nr = sqrtf(y0 * y0 + y1 * y1 + y2 * y2) + 1e-12f;
      const float h0 = y0 / nr, h1 = y1 / nr, h2 = y2 / nr;
      const float c = h0 * u0 + h1 * u1 + h2 * u2;
      l = 1.f - c;
      const float s = -inv_n / nr;
      g[0] = s * (u0 - c * h0);
      g[1] = s * (u1 - c * h1);
      g[2] = s * (u2 - c * h2);
    }
#pragma unroll
    for (int j = 0; j < kOut; ++j) dY[(size_t)m * kOut + j] = __float2bfloat16(g[j]);
  }
  // warp reduction of the loss
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) l += __shfl_down_sync(0xFFFFFFFFu, l, off);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss_sum, l);
}

// Column sums of a BF16 [M][N] matrix into g[n] (bias gradients).
__global__ void colsum_kernel(const bf16* __restrict__ D, int M, int N, float* __restrict__ g) {
  const int n = blockIdx.x * 32 + (threadIdx.x & 31);
  const int part = threadIdx.x >> 5;  // 8 row slices
  if (n >= N) return;
  float s = 0.f;
  for (int m = part; m < M; m += 8) s += __bfloat162float(D[(size_t)m * N + n]);
  atomicAdd(g + n, s);
}

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ mom,
                            float* __restrict__ vel, bf16* __restrict__ pb, bf16* __restrict__ pt, size_t n, float lr,
                            float b1, float b2, float c1, float c2, float eps) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float m = b1 * mom[i] + (1.f - b1) * gi;
    const float v = b2 * vel[i] + (1.f - b2) * gi * gi;
    mom[i] = m;
    vel[i] = v;
    const float x = p[i] - lr * (m / c1) / (sqrtf(v / c2) + eps);
    p[i] = x;
    const long long q = bf16_slot(i);
    if (q >= 0) pb[q] = __float2bfloat16(x);
    const long long t = tc_slot(i);
    if (t >= 0) pt[t] = __float2bfloat16(x);
  }
}

// BF16 copies of the weights: row-major (pb) and tensor-core operand layout (pt).
__global__ void to_bf16_kernel(const float* __restrict__ p, bf16* __restrict__ pb, bf16* __restrict__ pt, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const long long q = bf16_slot(i);
    if (q >= 0) pb[q] = __float2bfloat16(p[i]);
    const long long t = tc_slot(i);
    if (t >= 0) pt[t] = __float2bfloat16(p[i]);
  }
}

// ---------------------------------------------------------------- inference --

constexpr int kTile = 128;         // pairs per CTA tile
constexpr int kLd = kH + 8;        // shared-memory row stride (BF16 elements), 528 bytes
constexpr int kInferWarps = 16;    // 4 (rows) x 4 (columns) warps, 32 x 64 outputs each
constexpr size_t kInferSmem = (size_t)kTile * kLd * 2 + (size_t)kH * kLd * 2 + (size_t)kTile * kOut * 4;

// Copies a [rows][cols] BF16 matrix (cols a multiple of 8) into shared memory with row stride kLd.
__device__ __forceinline__ void stage_weights(bf16* dst, const bf16* __restrict__ src, int rows, int cols) {
  const int chunks = cols / 8;
  for (int idx = threadIdx.x; idx < rows * chunks; idx += blockDim.x) {
    const int r = idx / chunks, c = idx - r * chunks;
    *reinterpret_cast<uint4*>(dst + (size_t)r * kLd + 8 * c) =
        __ldg(reinterpret_cast<const uint4*>(src + (size_t)r * cols) + c);
  }
}

// acc (32 x 64 per warp) = act[rows of wm] (K columns) x W^T[cols of wn]
template <int K>
__device__ __forceinline__ void tile_product(const bf16* act, const bf16* w, float (&acc)[2][8][4], int wm, int wn,
                                             int gid, int tig) {
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;
#pragma unroll 4
  for (int kk = 0; kk < K; kk += 16) {
    uint32_t af[2][4];
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const bf16* a = act + (size_t)(wm * 32 + i * 16 + gid) * kLd + kk + 2 * tig;
      af[i][0] = ld_pair(a);
      af[i][1] = ld_pair(a + 8 * kLd);
      af[i][2] = ld_pair(a + 8);
      af[i][3] = ld_pair(a + 8 * kLd + 8);
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const bf16* bp = w + (size_t)(wn * 64 + j * 8 + gid) * kLd + kk + 2 * tig;
      uint32_t bfr[2] = {ld_pair(bp), ld_pair(bp + 8)};
      mma_bf16(acc[0][j], af[0], bfr);
      mma_bf16(acc[1][j], af[1], bfr);
    }
  }
}

__device__ __forceinline__ void tile_store_gelu(bf16* act, const float (&acc)[2][8][4], const float* __restrict__ bias,
                                                int wm, int wn, int gid, int tig) {
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int r = wm * 32 + i * 16 + gid;
      const int c = wn * 64 + j * 8 + 2 * tig;
      const float b0 = __ldg(bias + c), b1 = __ldg(bias + c + 1);
      __nv_bfloat162 lo, hi;
      lo.x = __float2bfloat16(gelu_fast(acc[i][j][0] + b0));
      lo.y = __float2bfloat16(gelu_fast(acc[i][j][1] + b1));
      hi.x = __float2bfloat16(gelu_fast(acc[i][j][2] + b0));
      hi.y = __float2bfloat16(gelu_fast(acc[i][j][3] + b1));
      *reinterpret_cast<__nv_bfloat162*>(act + (size_t)r * kLd + c) = lo;
      *reinterpret_cast<__nv_bfloat162*>(act + (size_t)(r + 8) * kLd + c) = hi;
    }
}

// One persistent CTA per SM; each 128-pair tile runs the four layers with the
// layer's weights staged in shared memory and the activations kept there.
// out: float[n][3], the unit direction (normalize) or the raw y.
__global__ void __launch_bounds__(kInferWarps * 32, 1)
    infer_kernel(const float4* __restrict__ pairs, uint32_t n, const bf16* __restrict__ wb,
                 const float* __restrict__ params, uint32_t n_classes, float* __restrict__ out, int normalize) {
  extern __shared__ __align__(16) unsigned char smem[];
  bf16* act = reinterpret_cast<bf16*>(smem);
  bf16* w = act + (size_t)kTile * kLd;
  float* yo = reinterpret_cast<float*>(w + (size_t)kH * kLd);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int wm = warp >> 2, wn = warp & 3;
  const int gid = lane >> 2, tig = lane & 3;
  const uint32_t n_tiles = (n + kTile - 1) / kTile;
  for (uint32_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    // features: four threads per row, eight columns each
    {
      const int r = tid >> 2, part = tid & 3;
      const uint32_t pid = tile * kTile + r;
      float q[16];
      uint32_t cls = 0;
      if (pid < n) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const float4 v = __ldg(pairs + 4 * (size_t)pid + j);
          q[4 * j] = v.x;
          q[4 * j + 1] = v.y;
          q[4 * j + 2] = v.z;
          q[4 * j + 3] = v.w;
        }
        cls = __float_as_uint(q[15]);
        if (cls >= n_classes) cls = 0;
      }
      const bf16* e = wb + qE + (size_t)cls * kEmb;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int c = 8 * part + j;
        act[(size_t)r * kLd + c] = __float2bfloat16(pid < n ? feature(q, e, c) : 0.f);
      }
    }
    stage_weights(w, wb + qW1, kH, kIn);
    __syncthreads();
    float acc[2][8][4];
    tile_product<kIn>(act, w, acc, wm, wn, gid, tig);
    __syncthreads();
    tile_store_gelu(act, acc, params + oB1, wm, wn, gid, tig);
    stage_weights(w, wb + qW2, kH, kH);
    __syncthreads();
    tile_product<kH>(act, w, acc, wm, wn, gid, tig);
    __syncthreads();
    tile_store_gelu(act, acc, params + oB2, wm, wn, gid, tig);
    stage_weights(w, wb + qW3, kH, kH);
    __syncthreads();
    tile_product<kH>(act, w, acc, wm, wn, gid, tig);
    __syncthreads();
    tile_store_gelu(act, acc, params + oB3, wm, wn, gid, tig);
    stage_weights(w, wb + qW4, kOut, kH);
    __syncthreads();
    // output layer: warps 0..7 each one 16-row slice, N = 8
    if (warp < kTile / 16) {
      float c4[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 4
      for (int kk = 0; kk < kH; kk += 16) {
        const bf16* a = act + (size_t)(warp * 16 + gid) * kLd + kk + 2 * tig;
        const uint32_t af[4] = {ld_pair(a), ld_pair(a + 8 * kLd), ld_pair(a + 8), ld_pair(a + 8 * kLd + 8)};
        const bf16* bp = w + (size_t)gid * kLd + kk + 2 * tig;
        const uint32_t bfr[2] = {ld_pair(bp), ld_pair(bp + 8)};
        mma_bf16(c4, af, bfr);
      }
      const int r = warp * 16 + gid, c = 2 * tig;
      const float b0 = __ldg(params + oB4 + c), b1 = __ldg(params + oB4 + c + 1);
      yo[r * kOut + c] = c4[0] + b0;
      yo[r * kOut + c + 1] = c4[1] + b1;
      yo[(r + 8) * kOut + c] = c4[2] + b0;
      yo[(r + 8) * kOut + c + 1] = c4[3] + b1;
    }
    __syncthreads();
    if (tid < kTile) {
      const uint32_t pid = tile * kTile + tid;
      if (pid < n) {
        float y0 = yo[tid * kOut], y1 = yo[tid * kOut + 1], y2 = yo[tid * kOut + 2];
        if (normalize) {
          const float s = y0 * y0 + y1 * y1 + y2 * y2;
          if (s > 0.f) {
            const float k = rsqrtf(s);
            y0 *= k;
            y1 *= k;
            y2 *= k;
          } else {
            y0 = 1.f;
            y1 = y2 = 0.f;
          }
        }
        out[3 * (size_t)pid] = y0;
        out[3 * (size_t)pid + 1] = y1;
        out[3 * (size_t)pid + 2] = y2;
      }
    }
    __syncthreads();
  }
}

}  // namespace wsm
}  // namespace fclg

using namespace fclg::wsm;

struct fclg_warmstart {
  int device = 0;
  int num_sms = 0;
  uint32_t n_classes = 0;
  size_t n_params = 0;
  std::string err;
  float* params = nullptr;  // FP32 master
  bf16* wb = nullptr;       // BF16 weights (row-major) + embedding
  bf16* wt = nullptr;       // BF16 weights in the tensor-core operand layout
  int* abort_flag = nullptr;  // set by an inference CTA whose bounded wait ran out
  float* grad = nullptr;
  float* mom = nullptr;
  float* vel = nullptr;
  uint64_t adam_t = 0;
  // training buffers for batches of up to cap rows
  uint32_t cap = 0;
  bf16 *X0 = nullptr, *A1 = nullptr, *A2 = nullptr, *A3 = nullptr, *dY = nullptr, *dZa = nullptr, *dZb = nullptr;
  float *Z1 = nullptr, *Z2 = nullptr, *Z3 = nullptr, *Y = nullptr, *loss = nullptr;
  uint32_t *cls = nullptr, *order = nullptr;
};

namespace {

int ws_fail(fclg_warmstart* w, int code, const std::string& msg) {
  if (w) w->err = msg;
  return code;
}

#define WS_CUDA(w, call)                                                                   \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) return ws_fail(w, FCLG_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
double uniform01(uint64_t& s) { return (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0); }

void free_train(fclg_warmstart* w) {
  void* bufs[] = {w->X0, w->A1, w->A2, w->A3, w->dY, w->dZa, w->dZb, w->Z1, w->Z2, w->Z3, w->Y, w->loss,
                  w->cls, w->order};
  for (void* p : bufs)
    if (p) cudaFree(p);
  w->X0 = w->A1 = w->A2 = w->A3 = w->dY = w->dZa = w->dZb = nullptr;
  w->Z1 = w->Z2 = w->Z3 = w->Y = w->loss = nullptr;
  w->cls = w->order = nullptr;
  w->cap = 0;
}

int ensure_train(fclg_warmstart* w, uint32_t rows) {
  const uint32_t M = (rows + 63) / 64 * 64;
  if (M <= w->cap) return FCLG_OK;
  free_train(w);
  const size_t h = (size_t)M * kH;
  WS_CUDA(w, cudaMalloc(&w->X0, (size_t)M * kIn * sizeof(bf16)));
  WS_CUDA(w, cudaMalloc(&w->A1, h * sizeof(bf16)));
  WS_CUDA(w, cudaMalloc(&w->A2, h * sizeof(bf16)));
  WS_CUDA(w, cudaMalloc(&w->A3, h * sizeof(bf16)));
  WS_CUDA(w, cudaMalloc(&w->dZa, h * sizeof(bf16)));
  WS_CUDA(w, cudaMalloc(&w->dZb, h * sizeof(bf16)));
  WS_CUDA(w, cudaMalloc(&w->dY, (size_t)M * kOut * sizeof(bf16)));
  WS_CUDA(w, cudaMalloc(&w->Z1, h * sizeof(float)));
  WS_CUDA(w, cudaMalloc(&w->Z2, h * sizeof(float)));
  WS_CUDA(w, cudaMalloc(&w->Z3, h * sizeof(float)));
  WS_CUDA(w, cudaMalloc(&w->Y, (size_t)M * kOut * sizeof(float)));
  WS_CUDA(w, cudaMalloc(&w->loss, sizeof(float)));
  WS_CUDA(w, cudaMalloc(&w->cls, (size_t)M * sizeof(uint32_t)));
  WS_CUDA(w, cudaMalloc(&w->order, (size_t)M * sizeof(uint32_t)));
  w->cap = M;
  return FCLG_OK;
}

template <class Epi>
cudaError_t gemm(const GemmArgs& g0, Epi epi, int splits, cudaStream_t st) {
  GemmArgs g = g0;
  if (splits < 1) splits = 1;
  g.k_chunk = ((g.K + splits - 1) / splits + 31) / 32 * 32;
  splits = (g.K + g.k_chunk - 1) / g.k_chunk;
  dim3 grid((g.N + 63) / 64, (g.M + 63) / 64, splits);
  gemm_kernel<Epi><<<grid, 128, 0, st>>>(g, epi);
  return cudaGetLastError();
}

GemmArgs nt(const bf16* X, int M, int K, const bf16* W, int N) {
  // C = X W^T: X [M][K] row-major, W [N][K] row-major
  return GemmArgs{X, K, 1, W, 1, K, M, N, K, 0};
}
GemmArgs nn(const bf16* D, int M, int N, const bf16* W, int K) {
  // C = D W: D [M][N] row-major (reduction over N), W [N][K] row-major
  return GemmArgs{D, N, 1, W, K, 1, M, K, N, 0};
}
GemmArgs tn(const bf16* D, int M, int N, const bf16* X, int K) {
  // C = D^T X: D [M][N], X [M][K] (reduction over M); C is [N][K]
  return GemmArgs{D, 1, N, X, K, 1, N, K, M, 0};
}

// Forward of rows [0, M) whose features are already in X0 (training layout).
int forward_train(fclg_warmstart* w, uint32_t M, cudaStream_t st) {
  const float* P = w->params;
  const bf16* B = w->wb;
  WS_CUDA(w, gemm(nt(w->X0, M, kIn, B + qW1, kH), EpiForward{P + oB1, w->Z1, w->A1, nullptr, kH, true}, 1, st));
  WS_CUDA(w, gemm(nt(w->A1, M, kH, B + qW2, kH), EpiForward{P + oB2, w->Z2, w->A2, nullptr, kH, true}, 1, st));
  WS_CUDA(w, gemm(nt(w->A2, M, kH, B + qW3, kH), EpiForward{P + oB3, w->Z3, w->A3, nullptr, kH, true}, 1, st));
  WS_CUDA(w, gemm(nt(w->A3, M, kH, B + qW4, kOut), EpiForward{P + oB4, nullptr, nullptr, w->Y, kOut, false}, 1, st));
  return FCLG_OK;
}

// Loss and gradient (into w->grad, zeroed here) of rows [0, n_valid) of a
// batch of M rows whose features are in X0.
int backward_train(fclg_warmstart* w, const float* labels, const uint32_t* order, uint32_t n_valid, uint32_t M,
                   cudaStream_t st) {
  const bf16* B = w->wb;
  float* G = w->grad;
  WS_CUDA(w, cudaMemsetAsync(G, 0, w->n_params * sizeof(float), st));
  loss_kernel<<<(M + 255) / 256, 256, 0, st>>>(w->Y, labels, order, n_valid, M, 1.f / (float)n_valid, w->dY,
                                                 w->loss);
  WS_CUDA(w, cudaGetLastError());
  const int splits = (int)std::max<uint32_t>(1, std::min<uint32_t>(32, M / 256));
  // layer 4
  WS_CUDA(w, gemm(tn(w->dY, M, kOut, w->A3, kH), EpiAccum{G + oW4, kH}, splits, st));
  colsum_kernel<<<1, 256, 0, st>>>(w->dY, M, kOut, G + oB4);
  WS_CUDA(w, gemm(nn(w->dY, M, kOut, B + qW4, kH), EpiBackGelu{w->Z3, w->dZa, kH}, 1, st));
  // layer 3
  WS_CUDA(w, gemm(tn(w->dZa, M, kH, w->A2, kH), EpiAccum{G + oW3, kH}, splits, st));
  colsum_kernel<<<kH / 32, 256, 0, st>>>(w->dZa, M, kH, G + oB3);
  WS_CUDA(w, gemm(nn(w->dZa, M, kH, B + qW3, kH), EpiBackGelu{w->Z2, w->dZb, kH}, 1, st));
  // layer 2
  WS_CUDA(w, gemm(tn(w->dZb, M, kH, w->A1, kH), EpiAccum{G + oW2, kH}, splits, st));
  colsum_kernel<<<kH / 32, 256, 0, st>>>(w->dZb, M, kH, G + oB2);
  WS_CUDA(w, gemm(nn(w->dZb, M, kH, B + qW2, kH), EpiBackGelu{w->Z1, w->dZa, kH}, 1, st));
  // layer 1 and the embedding
  WS_CUDA(w, gemm(tn(w->dZa, M, kH, w->X0, kIn), EpiAccum{G + oW1, kIn}, splits, st));
  colsum_kernel<<<kH / 32, 256, 0, st>>>(w->dZa, M, kH, G + oB1);
  WS_CUDA(w, gemm(nn(w->dZa, M, kH, B + qW1, kIn), EpiEmbed{w->cls, G + oE}, 1, st));
  return FCLG_OK;
}

int load_features(fclg_warmstart* w, const float4* pairs, const uint32_t* order, uint32_t n, uint32_t M,
                  cudaStream_t st) {
  features_kernel<<<(M + 127) / 128, 128, 0, st>>>(pairs, order, n, M, w->wb + qE, w->n_classes, w->X0, w->cls);
  WS_CUDA(w, cudaGetLastError());
  return FCLG_OK;
}

}  // namespace

namespace fclg {

namespace {

cudaError_t launch_infer(fclg_warmstart* w, const float4* pairs, uint32_t n, float* out, int normalize, bool legacy,
                         cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  (void)cudaGetLastError();  // a non-sticky error another caller left pending is not ours
  const uint32_t tiles = (n + kTile - 1) / kTile;
  const uint32_t blocks = std::min<uint32_t>(tiles, (uint32_t)w->num_sms);
  if (legacy)
    infer_kernel<<<blocks, kInferWarps * 32, kInferSmem, st>>>(pairs, n, w->wb, w->params, w->n_classes, out,
                                                               normalize);
  else
    infer_tc_kernel<<<blocks, kTcThreads, kTcSmem, st>>>(pairs, n, w->wt, w->wb, w->params, w->n_classes, out,
                                                         normalize, w->abort_flag);
  return cudaGetLastError();
}

}  // namespace

cudaError_t warmstart_predict(fclg_warmstart* w, const float4* pairs, uint32_t n, float* guess, cudaStream_t st) {
  return launch_infer(w, pairs, n, guess, 1, false, st);
}

int warmstart_device(const fclg_warmstart* w) { return w->device; }

}  // namespace fclg

extern "C" {

int fclg_warmstart_create(int device, uint32_t n_classes, uint32_t seed, fclg_warmstart** out) {
  if (!out) return FCLG_E_INVALID;
  *out = nullptr;
  if (n_classes == 0 || n_classes > (1u << 20)) return FCLG_E_INVALID;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) return FCLG_E_NO_DEVICE;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return FCLG_E_NO_DEVICE;
  if (prop.major * 10 + prop.minor != 103) return FCLG_E_NO_DEVICE;
  fclg_warmstart* w = new fclg_warmstart();
  w->device = device;
  w->num_sms = prop.multiProcessorCount;
  w->n_classes = n_classes;
  w->n_params = param_count(n_classes);
  // initialisation: weights and biases U(-1/sqrt(fan_in), 1/sqrt(fan_in)), embedding U(-1, 1)
  std::vector<float> h(w->n_params, 0.f);
  uint64_t s = 0x5EED0000ull + seed;
  auto fill = [&](size_t off, int rows, int cols, int used_rows, int used_cols, float bound) {
    for (int r = 0; r < rows; ++r)
      for (int c = 0; c < cols; ++c)
        h[off + (size_t)r * cols + c] =
            (r < used_rows && c < used_cols) ? (float)((2.0 * uniform01(s) - 1.0) * bound) : 0.f;
  };
  const float s1 = 1.f / std::sqrt((float)(kPoseCols + kEmb)), sh = 1.f / std::sqrt((float)kH);
  fill(oW1, kH, kIn, kH, kPoseCols + kEmb, s1);
  fill(oB1, 1, kH, 1, kH, s1);
  fill(oW2, kH, kH, kH, kH, sh);
  fill(oB2, 1, kH, 1, kH, sh);
  fill(oW3, kH, kH, kH, kH, sh);
  fill(oB3, 1, kH, 1, kH, sh);
  fill(oW4, kOut, kH, 3, kH, sh);
  fill(oB4, 1, kOut, 1, 3, sh);
  fill(oE, (int)n_classes, kEmb, (int)n_classes, kEmb, 1.f);
  const size_t nb = qE + (size_t)kEmb * n_classes;
  if (cudaSetDevice(device) != cudaSuccess || cudaMalloc(&w->params, w->n_params * 4) != cudaSuccess ||
      cudaMalloc(&w->wb, nb * sizeof(bf16)) != cudaSuccess || cudaMalloc(&w->grad, w->n_params * 4) != cudaSuccess ||
      cudaMalloc(&w->mom, w->n_params * 4) != cudaSuccess || cudaMalloc(&w->vel, w->n_params * 4) != cudaSuccess ||
      cudaMalloc(&w->wt, tTotal * sizeof(bf16)) != cudaSuccess || cudaMalloc(&w->abort_flag, sizeof(int)) != cudaSuccess ||
      cudaMemset(w->abort_flag, 0, sizeof(int)) != cudaSuccess ||
      cudaFuncSetAttribute(infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kInferSmem) !=
          cudaSuccess ||
      cudaFuncSetAttribute(infer_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem) !=
          cudaSuccess) {
    fclg_warmstart_destroy(w);
    return FCLG_E_CUDA;
  }
  if (fclg_warmstart_set_params(w, h.data(), w->n_params) != FCLG_OK) {
    fclg_warmstart_destroy(w);
    return FCLG_E_CUDA;
  }
  *out = w;
  return FCLG_OK;
}

void fclg_warmstart_destroy(fclg_warmstart* w) {
  if (!w) return;
  cudaSetDevice(w->device);
  free_train(w);
  void* bufs[] = {w->params, w->wb, w->wt, w->abort_flag, w->grad, w->mom, w->vel};
  for (void* p : bufs)
    if (p) cudaFree(p);
  delete w;
}

const char* fclg_warmstart_last_error(const fclg_warmstart* w) { return w ? w->err.c_str() : "null model"; }

uint64_t fclg_warmstart_param_count(const fclg_warmstart* w) { return w ? (uint64_t)w->n_params : 0; }

int fclg_warmstart_get_params(const fclg_warmstart* w, float* params, uint64_t n) {
  fclg_warmstart* m = const_cast<fclg_warmstart*>(w);
  if (!w || !params) return FCLG_E_INVALID;
  if (n != w->n_params) return ws_fail(m, FCLG_E_INVALID, "parameter count mismatch");
  WS_CUDA(m, cudaSetDevice(w->device));
  WS_CUDA(m, cudaMemcpy(params, w->params, n * 4, cudaMemcpyDeviceToHost));
  return FCLG_OK;
}

int fclg_warmstart_set_params(fclg_warmstart* w, const float* params, uint64_t n) {
  if (!w || !params) return FCLG_E_INVALID;
  if (n != w->n_params) return ws_fail(w, FCLG_E_INVALID, "parameter count mismatch");
  WS_CUDA(w, cudaSetDevice(w->device));
  WS_CUDA(w, cudaMemcpy(w->params, params, n * 4, cudaMemcpyHostToDevice));
  WS_CUDA(w, cudaMemset(w->wb, 0, (qE + (size_t)kEmb * w->n_classes) * sizeof(bf16)));
  WS_CUDA(w, cudaMemset(w->wt, 0, tTotal * sizeof(bf16)));
  to_bf16_kernel<<<256, 256>>>(w->params, w->wb, w->wt, w->n_params);
  WS_CUDA(w, cudaGetLastError());
  WS_CUDA(w, cudaMemset(w->mom, 0, n * 4));
  WS_CUDA(w, cudaMemset(w->vel, 0, n * 4));
  WS_CUDA(w, cudaDeviceSynchronize());
  w->adam_t = 0;
  return FCLG_OK;
}

int fclg_warmstart_predict(fclg_warmstart* w, const fclg_pair* d_pairs, uint32_t n, float* d_out, uint32_t flags,
                           void* stream) {
  if (!w) return FCLG_E_INVALID;
  if (n == 0) return FCLG_OK;
  if (!d_pairs || !d_out) return ws_fail(w, FCLG_E_INVALID, "null pair or output pointer");
  WS_CUDA(w, cudaSetDevice(w->device));
  WS_CUDA(w, fclg::launch_infer(w, reinterpret_cast<const float4*>(d_pairs), n, d_out,
                          (flags & FCLG_WS_NORMALIZE) ? 1 : 0, (flags & FCLG_WS_MMA_SYNC) != 0,
                          static_cast<cudaStream_t>(stream)));
  return FCLG_OK;
}

int fclg_warmstart_status(fclg_warmstart* w) {
  if (!w) return FCLG_E_INVALID;
  WS_CUDA(w, cudaSetDevice(w->device));
  WS_CUDA(w, cudaDeviceSynchronize());
  int e = 0;
  WS_CUDA(w, cudaMemcpy(&e, w->abort_flag, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) {
    WS_CUDA(w, cudaMemset(w->abort_flag, 0, sizeof(int)));
    return ws_fail(w, FCLG_E_CUDA, "a tensor-core inference CTA gave up a bounded wait; its directions are unset");
  }
  return FCLG_OK;
}

int fclg_warmstart_forward(fclg_warmstart* w, const fclg_pair* d_pairs, uint32_t n, float* d_y, void* stream) {
  if (!w) return FCLG_E_INVALID;
  if (n == 0) return FCLG_OK;
  if (!d_pairs || !d_y) return ws_fail(w, FCLG_E_INVALID, "null pair or output pointer");
  WS_CUDA(w, cudaSetDevice(w->device));
  (void)cudaGetLastError();  // not ours: left pending by another caller
  int rc = ensure_train(w, n);
  if (rc) return rc;
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  const uint32_t M = (n + 63) / 64 * 64;
  rc = load_features(w, reinterpret_cast<const float4*>(d_pairs), nullptr, n, M, st);
  if (rc) return rc;
  rc = forward_train(w, M, st);
  if (rc) return rc;
  WS_CUDA(w, cudaMemcpy2DAsync(d_y, 3 * sizeof(float), w->Y, kOut * sizeof(float), 3 * sizeof(float), n,
                               cudaMemcpyDeviceToDevice, st));
  return FCLG_OK;
}

int fclg_warmstart_gradient(fclg_warmstart* w, const fclg_pair* d_pairs, const float* d_labels, uint32_t n,
                            float* grad, float* loss) {
  if (!w) return FCLG_E_INVALID;
  if (!d_pairs || !d_labels || !grad || n == 0) return ws_fail(w, FCLG_E_INVALID, "bad gradient arguments");
  WS_CUDA(w, cudaSetDevice(w->device));
  (void)cudaGetLastError();  // not ours: left pending by another caller
  int rc = ensure_train(w, n);
  if (rc) return rc;
  const uint32_t M = (n + 63) / 64 * 64;
  rc = load_features(w, reinterpret_cast<const float4*>(d_pairs), nullptr, n, M, 0);
  if (rc) return rc;
  rc = forward_train(w, M, 0);
  if (rc) return rc;
  WS_CUDA(w, cudaMemset(w->loss, 0, sizeof(float)));
  rc = backward_train(w, d_labels, nullptr, n, M, 0);
  if (rc) return rc;
  WS_CUDA(w, cudaMemcpy(grad, w->grad, w->n_params * 4, cudaMemcpyDeviceToHost));
  float l = 0.f;
  WS_CUDA(w, cudaMemcpy(&l, w->loss, sizeof(float), cudaMemcpyDeviceToHost));
  if (loss) *loss = l / (float)n;
  return FCLG_OK;
}

int fclg_warmstart_train(fclg_warmstart* w, const fclg_pair* d_pairs, const float* d_labels, uint32_t n,
                         const fclg_train_config* cfg, float* epoch_loss) {
  if (!w) return FCLG_E_INVALID;
  if (!d_pairs || !d_labels || !cfg || n == 0) return ws_fail(w, FCLG_E_INVALID, "bad training arguments");
  const uint32_t batch = cfg->batch ? cfg->batch : 4096;
  const uint32_t epochs = cfg->epochs ? cfg->epochs : 1;
  const float lr0 = cfg->lr > 0.f ? cfg->lr : 1e-3f;
  const float lr1 = cfg->lr_final > 0.f ? cfg->lr_final : lr0 * 0.05f;
  if (batch % 64 != 0 || batch > (1u << 20)) return ws_fail(w, FCLG_E_INVALID, "batch must be a multiple of 64");
  WS_CUDA(w, cudaSetDevice(w->device));
  (void)cudaGetLastError();  // not ours: left pending by another caller
  int rc = ensure_train(w, batch);
  if (rc) return rc;
  cudaStream_t st = nullptr;
  WS_CUDA(w, cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  uint32_t* d_perm = nullptr;
  cudaError_t ce = cudaMalloc(&d_perm, (size_t)n * sizeof(uint32_t));
  if (ce != cudaSuccess) {
    cudaStreamDestroy(st);
    return ws_fail(w, FCLG_E_CUDA, std::string("cudaMalloc(perm): ") + cudaGetErrorString(ce));
  }
  std::vector<uint32_t> perm(n);
  for (uint32_t i = 0; i < n; ++i) perm[i] = i;
  uint64_t s = 0xC0FFEEull + cfg->seed;
  const uint64_t steps_total = (uint64_t)epochs * ((n + batch - 1) / batch);
  uint64_t step = 0;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  rc = FCLG_OK;
  for (uint32_t ep = 0; ep < epochs && rc == FCLG_OK; ++ep) {
    for (uint32_t i = n - 1; i > 0; --i) {
      const uint32_t j = (uint32_t)(splitmix(s) % (uint64_t)(i + 1));
      std::swap(perm[i], perm[j]);
    }
    ce = cudaMemcpyAsync(d_perm, perm.data(), (size_t)n * sizeof(uint32_t), cudaMemcpyHostToDevice, st);
    if (ce == cudaSuccess) ce = cudaMemsetAsync(w->loss, 0, sizeof(float), st);
    if (ce != cudaSuccess) { rc = ws_fail(w, FCLG_E_CUDA, cudaGetErrorString(ce)); break; }
    for (uint32_t b0 = 0; b0 < n && rc == FCLG_OK; b0 += batch, ++step) {
      const uint32_t nb = std::min(batch, n - b0);
      const uint32_t M = (nb + 63) / 64 * 64;
      rc = load_features(w, reinterpret_cast<const float4*>(d_pairs), d_perm + b0, nb, M, st);
      if (!rc) rc = forward_train(w, M, st);
      if (!rc) rc = backward_train(w, d_labels, d_perm + b0, nb, M, st);
      if (rc) break;
      // cosine learning-rate decay from lr0 to lr1
      const double f = steps_total > 1 ? (double)step / (double)(steps_total - 1) : 1.0;
      const float lr = (float)(lr1 + 0.5 * (lr0 - lr1) * (1.0 + std::cos(3.14159265358979 * f)));
      w->adam_t += 1;
      const float c1 = 1.f - std::pow(b1, (float)w->adam_t), c2 = 1.f - std::pow(b2, (float)w->adam_t);
      adam_kernel<<<512, 256, 0, st>>>(w->params, w->grad, w->mom, w->vel, w->wb, w->wt, w->n_params, lr, b1, b2,
                                       c1, c2, eps);
      ce = cudaGetLastError();
      if (ce != cudaSuccess) rc = ws_fail(w, FCLG_E_CUDA, cudaGetErrorString(ce));
    }
    if (rc) break;
    float l = 0.f;
    ce = cudaMemcpyAsync(&l, w->loss, sizeof(float), cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) { rc = ws_fail(w, FCLG_E_CUDA, cudaGetErrorString(ce)); break; }
    if (epoch_loss) epoch_loss[ep] = l / (float)n;
  }
  cudaStreamSynchronize(st);
  cudaFree(d_perm);
  cudaStreamDestroy(st);
  return rc;
}

}  // extern "C"
