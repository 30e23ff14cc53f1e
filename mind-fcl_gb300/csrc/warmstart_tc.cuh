// Warm-start inference on the 5th-generation tensor cores (tcgen05), included
// by warmstart.cu after the model constants.
//
// One persistent CTA of sixteen warps per SM; each tile is 128 pairs (the
// MMA's M).  Per tile:
//   features -> act (shared, BF16)                        all threads
//   per layer: D (TMEM, FP32, 128 lanes x N columns) = act x W^T
//              by tcgen05.mma kind::f16 issued by one thread, operands read
//              from shared memory through matrix descriptors
//   epilogue:  tcgen05.ld of 64 columns of the thread's row (four warps per
//              TMEM lane quarter), + bias (staged in shared memory once),
//              GELU, BF16 -> act
// Weights stream from global memory (already in the MMA's K-major
// core-matrix layout, see tc_slot) into two 64 KB buffers with cp.async.bulk
// on mbarrier transaction counts: W1 | W2 (two N halves) | W3 (two halves) |
// W4.  A chunk loads as soon as its buffer is free -- right after the MMAs
// that read the buffer complete -- so the loads run under the epilogues and
// under the other buffer's MMAs.
//
// Shared-memory operand layout (K-major, no swizzle): 8 x 16-byte core
// matrices (8 rows x 8 BF16 along K, 128 contiguous bytes); along K the core
// matrices are 128 bytes apart (leading byte offset), along M / N the 8-row
// groups are 4096 bytes apart (stride byte offset; 512 for W1, K = 32).
//
// Every wait is bounded by a clock budget; a wait that runs out sets the
// CTA's abort flag, the CTA drains its copies and MMAs in flight (bounded),
// frees its TMEM, records the failure in *err and returns.
#pragma once

namespace fclg {
namespace wsm {

constexpr int kTcThreads = 512;  // 16 warps: warp w reads TMEM lane quarter w % 4, columns 64 (w / 4) ..
constexpr uint32_t kTcCols = 256;                      // TMEM columns: one 128 x 256 FP32 accumulator
constexpr uint32_t kActBytes = 128u * kH * 2u;         // 64 KB
constexpr uint32_t kBufBytes = 65536u;
constexpr uint32_t kGroupStride = 4096u;               // 32 core matrices of 128 bytes along K
constexpr size_t kTcBiasOffset = (size_t)kActBytes + 2 * kBufBytes + 128;  // b1 | b2 | b3, FP32
constexpr size_t kTcSmem = kTcBiasOffset + 3 * (size_t)kH * 4;
constexpr long long kWaitCycles = 1ll << 31;           // about one second per wait

// tc-layout weight copy (BF16 elements): W1 [256][32] | W2 [256][256] | W3 | W4 padded to 16 rows
constexpr size_t tW1 = 0, tW2 = tW1 + (size_t)kH * kIn, tW3 = tW2 + (size_t)kH * kH, tW4 = tW3 + (size_t)kH * kH;
constexpr size_t tTotal = tW4 + (size_t)16 * kH;

__host__ __device__ inline size_t core_offset(int n, int k, int kchunks) {
  return (size_t)(n >> 3) * (size_t)(kchunks * 64) + (size_t)(k >> 3) * 64 + (size_t)(n & 7) * 8 + (size_t)(k & 7);
}

// tc-layout slot of master parameter i (weights only), or -1.
__device__ __forceinline__ long long tc_slot(size_t i) {
  if (i < oB1) return (long long)(tW1 + core_offset((int)(i / kIn), (int)(i % kIn), kIn / 8));
  if (i >= oW2 && i < oB2) return (long long)(tW2 + core_offset((int)((i - oW2) / kH), (int)((i - oW2) % kH), 32));
  if (i >= oW3 && i < oB3) return (long long)(tW3 + core_offset((int)((i - oW3) / kH), (int)((i - oW3) % kH), 32));
  if (i >= oW4 && i < oB4) return (long long)(tW4 + core_offset((int)((i - oW4) / kH), (int)((i - oW4) % kH), 32));
  return -1;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor: start address, leading / stride byte
// offsets (all >> 4), descriptor version 1 (bits 46-47), no swizzle.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
         (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), BF16 A
// and B (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t umma_idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t phase) {
  uint32_t done;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(bar), "r"(phase)
      : "memory");
  return done != 0;
}

// Bounded wait for the completion of phase `phase`; false when the clock
// budget runs out (the abort flag is then set) or, with honour_abort, when
// another thread has aborted.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t phase, volatile int* abort, bool honour_abort) {
  const long long t0 = clock64();
  while (!mbar_try(bar, phase)) {
    if (honour_abort && *abort) return false;
    if (clock64() - t0 > kWaitCycles) {
      *abort = 1;
      return false;
    }
  }
  return true;
}

__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

__device__ __forceinline__ void umma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

__device__ __forceinline__ void tmem_ld16(uint32_t addr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
        "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(addr)
      : "memory");
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&h);
}

// Columns [cbeg, cbeg + 64) of row r of a 128 x 256 FP32 accumulator (TMEM
// row address trow) -> + bias (shared memory), GELU, BF16 -> act in the
// operand layout.
__device__ __forceinline__ void tc_epilogue_hidden(uint32_t trow, const float* bias, unsigned char* act, int r,
                                                   int cbeg) {
  unsigned char* row = act + (size_t)(r >> 3) * kGroupStride + (size_t)(r & 7) * 16;
#pragma unroll 1
  for (int c0 = cbeg; c0 < cbeg + 64; c0 += 32) {
    uint32_t v0[16], v1[16];
    tmem_ld16(trow + (uint32_t)c0, v0);
    tmem_ld16(trow + (uint32_t)c0 + 16u, v1);
    float bv[32];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const float4 t = reinterpret_cast<const float4*>(bias + c0)[q];
      bv[4 * q] = t.x;
      bv[4 * q + 1] = t.y;
      bv[4 * q + 2] = t.z;
      bv[4 * q + 3] = t.w;
    }
    tmem_wait_ld();
    uint32_t p[16];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      p[j] = pack_bf16(gelu_fast(__uint_as_float(v0[2 * j]) + bv[2 * j]),
                       gelu_fast(__uint_as_float(v0[2 * j + 1]) + bv[2 * j + 1]));
      p[8 + j] = pack_bf16(gelu_fast(__uint_as_float(v1[2 * j]) + bv[16 + 2 * j]),
                           gelu_fast(__uint_as_float(v1[2 * j + 1]) + bv[16 + 2 * j + 1]));
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
      *reinterpret_cast<uint4*>(row + (size_t)((c0 >> 3) + q) * 128) =
          make_uint4(p[4 * q], p[4 * q + 1], p[4 * q + 2], p[4 * q + 3]);
  }
}

__global__ void __launch_bounds__(kTcThreads, 1)
    infer_tc_kernel(const float4* __restrict__ pairs, uint32_t n, const bf16* __restrict__ wt,
                    const bf16* __restrict__ wb, const float* __restrict__ params, uint32_t n_classes,
                    float* __restrict__ out, int normalize, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  unsigned char* act = tc_smem;
  unsigned char* buf0 = tc_smem + kActBytes;
  unsigned char* buf1 = buf0 + kBufBytes;
  uint64_t* bars = reinterpret_cast<uint64_t*>(buf1 + kBufBytes);  // full0, full1, mma, half, drain
  uint32_t* s_taddr = reinterpret_cast<uint32_t*>(bars + 5);
  volatile int* s_abort = reinterpret_cast<volatile int*>(bars + 6);
  float* s_bias = reinterpret_cast<float*>(tc_smem + kTcBiasOffset);
  const int tid = threadIdx.x, warp = tid >> 5;
  const bool leader = tid == 0;
  const int row = (warp & 3) * 32 + (tid & 31);  // TMEM lane (tile row) this thread reads
  const int cbeg = (warp >> 2) * 64;              // its 64 accumulator columns
  const uint32_t bar_full[2] = {smem_u32(&bars[0]), smem_u32(&bars[1])};
  const uint32_t bar_mma = smem_u32(&bars[2]), bar_half = smem_u32(&bars[3]), bar_drain = smem_u32(&bars[4]);
  const uint32_t a_act = smem_u32(act);
  const uint32_t a_buf[2] = {smem_u32(buf0), smem_u32(buf1)};
  if (leader) {
    for (int i = 0; i < 5; ++i) mbar_init(smem_u32(&bars[i]), 1);
    *s_abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  for (int i = tid; i < 3 * kH; i += kTcThreads) {
    const size_t base = i < kH ? oB1 : (i < 2 * kH ? oB2 : oB3);
    s_bias[i] = params[base + (size_t)(i % kH)];
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(s_taddr)),
                 "r"(kTcCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t taddr = *s_taddr;
  const uint32_t trow = taddr + ((uint32_t)((warp & 3) * 32) << 16);  // this warp's TMEM lane quarter

  const char* src = reinterpret_cast<const char*>(wt);
  const char* srcW1 = src + tW1 * 2;
  const char* srcW2 = src + tW2 * 2;
  const char* srcW3 = src + tW3 * 2;
  const char* srcW4 = src + tW4 * 2;
  constexpr uint32_t id256 = umma_idesc(128, 256), id128 = umma_idesc(128, 128), id16 = umma_idesc(128, 16);

  uint32_t ph_full[2] = {0u, 0u}, ph_mma = 0u, ph_half = 0u;
  bool pending[2] = {false, false};
  auto load = [&](int b, const char* s, uint32_t bytes) {
    bulk_load(a_buf[b], s, bytes, bar_full[b]);
    pending[b] = true;
  };
  auto wait_full = [&](int b) {
    if (!mbar_wait(bar_full[b], ph_full[b], s_abort, true)) return false;
    ph_full[b] ^= 1u;
    pending[b] = false;
    return true;
  };
  // D (columns d0..) += act[:, 0:K] x W^T from buffer b, K / 16 MMAs
  auto mma_layer = [&](uint32_t d0, int b, int ksteps, uint32_t sbo_b, uint32_t idesc) {
    for (int s = 0; s < ksteps; ++s)
      umma(taddr + d0, umma_desc(a_act + (uint32_t)s * 256u, 128u, kGroupStride),
           umma_desc(a_buf[b] + (uint32_t)s * 256u, 128u, sbo_b), idesc, s > 0 ? 1u : 0u);
  };
  // all threads; the result is warp-uniform (the TMEM loads that follow are .sync.aligned)
  auto all_wait_mma = [&]() {
    const bool ok = mbar_wait(bar_mma, ph_mma, s_abort, true);
    if (ok) ph_mma ^= 1u;
    tc_fence_after();
    return __all_sync(0xFFFFFFFFu, ok) != 0;
  };
  auto end_stage = [&]() {
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
  };

  const uint32_t n_tiles = (n + 127) / 128;
  if (leader && blockIdx.x < n_tiles) {
    load(0, srcW1, (uint32_t)(kH * kIn * 2));
    load(1, srcW2, kBufBytes);
  }
  for (uint32_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const bool more = tile + gridDim.x < n_tiles;
    // features: four threads per row, one 8-column chunk each
    {
      const int fr = tid >> 2, chunk = tid & 3;
      const uint32_t pid = tile * 128 + (uint32_t)fr;
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
      uint32_t p[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int c = 8 * chunk + 2 * j;
        p[j] = pid < n ? pack_bf16(feature(q, e, c), feature(q, e, c + 1)) : 0u;
      }
      unsigned char* dst = act + (size_t)(fr >> 3) * kGroupStride + (size_t)chunk * 128 + (size_t)(fr & 7) * 16;
      *reinterpret_cast<uint4*>(dst) = make_uint4(p[0], p[1], p[2], p[3]);
    }
    end_stage();
    if (*s_abort) break;

    // layer 1: K = 32, N = 256 (W1 in buffer 0; W2's first half is in or on its way to buffer 1)
    if (leader && wait_full(0)) {
      tc_fence_after();
      mma_layer(0, 0, kIn / 16, 512u, id256);
      umma_commit(bar_mma);
    }
    const bool ok1 = all_wait_mma();
    if (leader && ok1) load(0, srcW2 + kBufBytes, kBufBytes);  // buffer 0 is free: W2's second half
    if (ok1) tc_epilogue_hidden(trow, s_bias, act, row, cbeg);
    end_stage();
    if (*s_abort) break;

    // layers 2 and 3: two N halves each, weights double-buffered
    for (int layer = 2; layer <= 3; ++layer) {
      if (leader) {
        if (wait_full(1)) {
          mma_layer(0, 1, kH / 16, kGroupStride, id128);
          umma_commit(bar_half);
        }
        if (!*s_abort && wait_full(0)) {
          mma_layer(128, 0, kH / 16, kGroupStride, id128);
          umma_commit(bar_mma);
        }
        // buffer 1 is free once the first half's MMAs completed: next chunk
        if (!*s_abort && mbar_wait(bar_half, ph_half, s_abort, true)) {
          ph_half ^= 1u;
          if (layer == 2) load(1, srcW3, kBufBytes);
          else load(1, srcW4, (uint32_t)(16 * kH * 2));
        }
      }
      const bool okl = all_wait_mma();
      // buffer 0 is free (the layer's MMAs completed): W3's second half, or the next tile's W1
      if (leader && okl) {
        if (layer == 2) load(0, srcW3 + kBufBytes, kBufBytes);
        else if (more) load(0, srcW1, (uint32_t)(kH * kIn * 2));
      }
      if (okl) tc_epilogue_hidden(trow, s_bias + (layer - 1) * kH, act, row, cbeg);
      end_stage();
      if (*s_abort) break;
    }
    if (*s_abort) break;

    // layer 4: N = 16 (rows 3..15 of W4 are zero)
    if (leader && wait_full(1)) {
      mma_layer(0, 1, kH / 16, kGroupStride, id16);
      umma_commit(bar_mma);
    }
    const bool ok4 = all_wait_mma();
    if (leader && ok4 && more) load(1, srcW2, kBufBytes);  // buffer 1 is free: the next tile's W2 first half
    if (ok4 && warp < 4) {
      uint32_t v[16];
      tmem_ld16(trow, v);
      tmem_wait_ld();
      const uint32_t pid = tile * 128 + (uint32_t)row;
      if (pid < n) {
        float y0 = __uint_as_float(v[0]) + __ldg(params + oB4);
        float y1 = __uint_as_float(v[1]) + __ldg(params + oB4 + 1);
        float y2 = __uint_as_float(v[2]) + __ldg(params + oB4 + 2);
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
    end_stage();
    if (*s_abort) break;
  }

  // drain (only reached with work in flight after an abort) and free TMEM
  if (leader && *s_abort) {
    for (int b = 0; b < 2; ++b)
      if (pending[b]) mbar_wait(bar_full[b], ph_full[b], s_abort, false);
    umma_commit(bar_drain);  // tracks every MMA this thread issued
    mbar_wait(bar_drain, 0u, s_abort, false);
    atomicExch(err, 1);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(kTcCols) : "memory");
}

}  // namespace wsm
}  // namespace fclg
