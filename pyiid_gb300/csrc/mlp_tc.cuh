// The surrogate's per-atom MLP (32 -> 128 -> 128 -> 1, SiLU) forward and
// descriptor gradient on the fifth-generation tensor cores:
//   z1 = X W1 + b1, h1 = silu(z1), z2 = h1 W2 + b2, y = silu(z2) . w3 + b3,
//   dE/dX = ((w3 * silu'(z2)) W2^T * silu'(z1)) W1^T      (E = sum_a y_a)
// with BF16 operands and FP32 accumulation, the same roundings as the
// register-resident mma.sync kernel (mlp_fused_kernel): activations are
// rounded to BF16 where they become the next product's operand.
//
// One persistent CTA per SM, 128 threads, 128 atoms per tile (thread r =
// row r = tensor-memory lane r).  The four weight operands are staged once
// per CTA in shared memory as K-major blocks in the 128-byte swizzled order
// the shared-memory descriptors read (64 BF16 per row); per tile:
//   X  -> smem            tcgen05.mma  z1 = X W1          (N 128, K 32)
//   z1 -> h1 -> smem      tcgen05.mma  z2 = h1 W2         (N 128, K 128)
//   z2 -> y, g2 -> smem   tcgen05.mma  gh1 = g2 W2^T      (N 128, K 128)
//   gh1, z1 -> g1 -> smem tcgen05.mma  gX = g1 W1^T       (N 32,  K 128)
//   gX -> FP16 rows
// Thread 0 issues each product (4, 8, 8 and 8 instructions of K 16) and
// commits it to one mbarrier; every thread reads its row back with
// tcgen05.ld.  Tensor memory: 256 columns (z1 in 0..127, z2 and then gh1
// in 128..255, gX in 0..31 once z1 is consumed).  Threads' shared-memory
// stores reach the tensor core's reads through fence.proxy.async before
// the barrier that precedes the product.  Every wait is bounded (~1 s):
// on time-out the CTA records an error in *err and stops.
//
// Measured on 64 x 1,000 atoms: 151 us against 70 us for the register-
// resident mma.sync kernel (launch variant 0; this is variant 1).  The
// products are small (tensor pipe busy 1.7 % of the time); the SiLU and
// SiLU' epilogues run one thread per row on 4 warps per SM at 15 % issue,
// where the mma.sync kernel spreads them over 16 warps.  mlp_tc2_kernel
// below (variant 2, the default) keeps two tiles in flight per CTA with two
// threads per row: 57 us.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "umma_gemm.cuh"

namespace pyiid {
namespace mlptc {

using namespace umma;

constexpr int kRows = 128;  // atoms per tile
constexpr int kIn = 32, kHid = 128;
constexpr int kBlk = kRows * 128;  // bytes of one 128-row K block

// byte offsets from the 1024-aligned base of dynamic shared memory
constexpr int kOffW1T = 0;                    // [h 128][c 32]   16 KB
constexpr int kOffW2T = kOffW1T + kBlk;       // 2 x [o 128][i 64] 32 KB
constexpr int kOffW2 = kOffW2T + 2 * kBlk;    // 2 x [i 128][o 64] 32 KB
constexpr int kOffW1 = kOffW2 + 2 * kBlk;     // 2 x [c 32][h 64]   8 KB
constexpr int kOffX = kOffW1 + 2 * 32 * 128;  // [row 128][c 32]   16 KB
constexpr int kOffAct = kOffX + kBlk;         // 2 x [row][64]     32 KB
constexpr int kOffVec = kOffAct + 2 * kBlk;   // b1, b2, w3 (FP32)
constexpr int kOffBar = kOffVec + 3 * kHid * 4;
constexpr int kSmemBytes = kOffBar + 16 + 1024;  // + alignment slack
static_assert(kSmemBytes <= 232448, "shared memory per CTA");

// byte offset of element (r, k), k < 64, of a K-major BF16 block
__device__ __forceinline__ int bf16_at(int r, int k) {
  return r * 128 + ((((k >> 3) ^ (r & 7))) << 4) + ((k & 7) << 1);
}

// 16-byte chunk c (8 BF16, k = 8c .. 8c + 7) of row r
__device__ __forceinline__ int chunk_at(int r, int c) {
  return r * 128 + ((c ^ (r & 7)) << 4);
}

__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  const __nv_bfloat16 l = __float2bfloat16_rn(lo), h = __float2bfloat16_rn(hi);
  return (uint32_t)__bfloat16_as_ushort(l) |
         ((uint32_t)__bfloat16_as_ushort(h) << 16);
}

__device__ __forceinline__ float silu(float x) { return x / (1.f + __expf(-x)); }
__device__ __forceinline__ float dsilu(float x) {
  const float s = 1.f / (1.f + __expf(-x));
  return s * (1.f + x * (1.f - s));
}

// 32 FP32 values -> 4 chunks of BF16 in row r of a K-major block pair,
// columns k0 .. k0 + 31 (k0 a multiple of 32)
__device__ __forceinline__ void store_row32(unsigned char *blocks, int r,
                                            int k0, const float (&v)[32]) {
  unsigned char *blk = blocks + (k0 >> 6) * kBlk;
  const int c0 = (k0 & 63) >> 3;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    uint4 w;
    w.x = pack_bf16x2(v[8 * c + 0], v[8 * c + 1]);
    w.y = pack_bf16x2(v[8 * c + 2], v[8 * c + 3]);
    w.z = pack_bf16x2(v[8 * c + 4], v[8 * c + 5]);
    w.w = pack_bf16x2(v[8 * c + 6], v[8 * c + 7]);
    *reinterpret_cast<uint4 *>(blk + chunk_at(r, c0 + c)) = w;
  }
}

__global__ void __launch_bounds__(128, 1)
    mlp_tc_kernel(const __nv_bfloat16 *__restrict__ X, int n_atoms,
                  const __nv_bfloat16 *__restrict__ W1,
                  const float *__restrict__ b1,
                  const __nv_bfloat16 *__restrict__ W2,
                  const float *__restrict__ b2, const float *__restrict__ w3,
                  const float *__restrict__ b3, float *__restrict__ y,
                  __half *__restrict__ gout, int *err) {
  extern __shared__ unsigned char smem_raw[];
  const uint32_t raw = smem_addr(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  unsigned char *sp = smem_raw + (base - raw);
  float *sb1 = reinterpret_cast<float *>(sp + kOffVec);
  float *sb2 = sb1 + kHid, *sw3 = sb2 + kHid;
  const uint32_t bar = base + kOffBar;
  uint32_t *slot = reinterpret_cast<uint32_t *>(sp + kOffBar + 8);
  const int tid = threadIdx.x, warp = tid >> 5;

  // weights, as K-major operands: W1 [c][h] and W2 [i][o] are row-major
  for (int e = tid; e < kIn * kHid; e += blockDim.x) {
    const int c = e / kHid, h = e % kHid;
    const __nv_bfloat16 v = W1[e];
    // layer 1 B: row h, k = c;  gX B: row c, k = h (two K blocks)
    *reinterpret_cast<__nv_bfloat16 *>(sp + kOffW1T + bf16_at(h, c)) = v;
    *reinterpret_cast<__nv_bfloat16 *>(sp + kOffW1 + (h >> 6) * (32 * 128) +
                                       bf16_at(c, h & 63)) = v;
  }
  for (int e = tid; e < kHid * kHid; e += blockDim.x) {
    const int i = e / kHid, o = e % kHid;
    const __nv_bfloat16 v = W2[e];
    // layer 2 B: row o, k = i;  gh1 B: row i, k = o
    *reinterpret_cast<__nv_bfloat16 *>(sp + kOffW2T + (i >> 6) * kBlk +
                                       bf16_at(o, i & 63)) = v;
    *reinterpret_cast<__nv_bfloat16 *>(sp + kOffW2 + (o >> 6) * kBlk +
                                       bf16_at(i, o & 63)) = v;
  }
  for (int e = tid; e < kHid; e += blockDim.x) {
    sb1[e] = b1[e];
    sb2[e] = b2[e];
    sw3[e] = w3[e];
  }
  if (tid == 0) {
    mbar_init(bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncwarp();
  if (warp == 0) {
    asm volatile(
        "tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n"
        ::"r"(smem_addr(slot)), "r"(256)
        : "memory");
    asm volatile(
        "tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::
            : "memory");
  }
  fence_proxy_async();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *slot;
  const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
  const float bias3 = b3[0];
  const int n_tiles = (n_atoms + kRows - 1) / kRows;
  uint32_t phase = 0;
  unsigned char *act = sp + kOffAct;

  // issue one product chain: A blocks at a_off (kb blocks of kBlk), B
  // blocks at b_off (b_blk bytes apart), n_k K-steps of 16
  auto product = [&](uint32_t d, int a_off, int b_off, int b_blk, int n_k,
                     uint32_t idesc) {
    tc_fence_after();
    for (int s = 0; s < n_k; ++s) {
      const int kb = s >> 2, j = s & 3;
      const uint64_t da = sdesc(base + a_off + kb * kBlk + 32 * j);
      const uint64_t db = sdesc(base + b_off + kb * b_blk + 32 * j);
      mma_f16(d, da, db, idesc, s != 0);
    }
    mma_commit(bar);
  };
  // all threads: wait for the last product; false on time-out (every
  // thread then leaves the tile loop together)
  auto wait_product = [&]() {
    const bool ok = mbar_wait(bar, phase & 1);
    ++phase;
    const bool bad = __syncthreads_or(!ok);
    tc_fence_after();
    return !bad;
  };

  for (int t = blockIdx.x; t < n_tiles; t += gridDim.x) {
    const int row = t * kRows + tid;
    const bool have = row < n_atoms;
    // X row (32 BF16 = 4 chunks)
    {
      const uint4 *xr = reinterpret_cast<const uint4 *>(X + (size_t)row * kIn);
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const uint4 w = have ? xr[c] : make_uint4(0u, 0u, 0u, 0u);
        *reinterpret_cast<uint4 *>(sp + kOffX + chunk_at(tid, c)) = w;
      }
    }
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    if (tid == 0)
      product(tmem, kOffX, kOffW1T, 0, kIn / 16, idesc_bf16(kRows, kHid));
    if (!wait_product()) break;

    // h1 = silu(z1 + b1) -> act
#pragma unroll 1
    for (int c0 = 0; c0 < kHid; c0 += 32) {
      float v[32];
      tmem_ld32(tmem + lane_base + (uint32_t)c0, v);
#pragma unroll
      for (int k = 0; k < 32; ++k) v[k] = silu(v[k] + sb1[c0 + k]);
      store_row32(act, tid, c0, v);
    }
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    if (tid == 0)
      product(tmem + 128, kOffAct, kOffW2T, kBlk, kHid / 16,
              idesc_bf16(kRows, kHid));
    if (!wait_product()) break;

    // y and g2 = w3 * silu'(z2 + b2) -> act
    float yr = bias3;
#pragma unroll 1
    for (int c0 = 0; c0 < kHid; c0 += 32) {
      float v[32];
      tmem_ld32(tmem + 128 + lane_base + (uint32_t)c0, v);
#pragma unroll
      for (int k = 0; k < 32; ++k) {
        const float u = v[k] + sb2[c0 + k];
        yr = fmaf(silu(u), sw3[c0 + k], yr);
        v[k] = sw3[c0 + k] * dsilu(u);
      }
      store_row32(act, tid, c0, v);
    }
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    if (tid == 0)
      product(tmem + 128, kOffAct, kOffW2, kBlk, kHid / 16,
              idesc_bf16(kRows, kHid));
    if (!wait_product()) break;

    // g1 = gh1 * silu'(z1 + b1) -> act
#pragma unroll 1
    for (int c0 = 0; c0 < kHid; c0 += 32) {
      float v[32], z[32];
      tmem_ld32(tmem + 128 + lane_base + (uint32_t)c0, v);
      tmem_ld32(tmem + lane_base + (uint32_t)c0, z);
#pragma unroll
      for (int k = 0; k < 32; ++k) v[k] *= dsilu(z[k] + sb1[c0 + k]);
      store_row32(act, tid, c0, v);
    }
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    if (tid == 0)
      product(tmem, kOffAct, kOffW1, 32 * 128, kHid / 16,
              idesc_bf16(kRows, kIn));
    if (!wait_product()) break;

    // gX -> FP16 row, y
    {
      float v[32];
      tmem_ld32(tmem + lane_base, v);
      if (have) {
        uint4 *gr = reinterpret_cast<uint4 *>(gout + (size_t)row * kIn);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          uint4 w;
          const __half2 h0 = __floats2half2_rn(v[8 * c + 0], v[8 * c + 1]);
          const __half2 h1 = __floats2half2_rn(v[8 * c + 2], v[8 * c + 3]);
          const __half2 h2 = __floats2half2_rn(v[8 * c + 4], v[8 * c + 5]);
          const __half2 h3 = __floats2half2_rn(v[8 * c + 6], v[8 * c + 7]);
          w.x = *reinterpret_cast<const uint32_t *>(&h0);
          w.y = *reinterpret_cast<const uint32_t *>(&h1);
          w.z = *reinterpret_cast<const uint32_t *>(&h2);
          w.w = *reinterpret_cast<const uint32_t *>(&h3);
          gr[c] = w;
        }
        y[row] = yr;
      }
    }
    // the next tile's first product overwrites z1 / gX and X
    tc_fence_before();
    __syncthreads();
  }
  if (tid == 0 && phase != 4u * (uint32_t)((n_tiles - (int)blockIdx.x +
                                            (int)gridDim.x - 1) /
                                           (int)gridDim.x)) {
    atomicCAS(err, 0, kErrAccumWait);
    // a product that timed out may still be writing tensor memory: one more
    // bounded wait for its commit before the columns are freed
    mbar_wait(bar, (phase - 1u) & 1u);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(
                     tmem),
                 "r"(256)
                 : "memory");
  }
}

// Two tiles in flight, two threads per row (launch variant 2).  512 threads
// in two slots of 8 warps; slot s takes tiles 2 blockIdx.x + s, + 2
// gridDim.x, ... with its own X and activation blocks, its own 256 tensor-
// memory columns, mbarrier and named barrier, so one slot's epilogues run
// while the other's product is in flight.  Warp w of a slot reads lane
// quarter w mod 4 (rows 32 (w mod 4) ..) and column half (w / 4) mod 2 of
// every 128-column result; the layer-2 output y is the fixed-order sum of
// the halves' partial dot products (bias on half 0).  The weights are staged
// once per CTA for both slots.  Each slot's wait is bounded; a time-out ends
// that slot's loop for all its threads (bar.red.or over the slot) and is
// recorded in *err.
constexpr int kSlotBytes = 3 * kBlk;               // X + 2 activation blocks
constexpr int kOffSlots = kOffX;                   // after the weights
constexpr int kOffVec2 = kOffSlots + 2 * kSlotBytes;
constexpr int kOffY2 = kOffVec2 + 3 * kHid * 4;    // [slot][half][row] FP32
constexpr int kOffBar2 = kOffY2 + 2 * 2 * kRows * 4;
constexpr int kSmemBytes2 = kOffBar2 + 32 + 1024;  // + alignment slack
static_assert(kSmemBytes2 <= 232448, "shared memory per CTA");
static_assert(kOffSlots % 1024 == 0 && kSlotBytes % 1024 == 0,
              "operand blocks 1024-byte aligned");

__device__ __forceinline__ void slot_sync(int id) {
  asm volatile("bar.sync %0, 256;\n" ::"r"(id) : "memory");
}
// barrier over the slot's 256 threads; true if any thread passed true
__device__ __forceinline__ bool slot_sync_or(int id, bool v) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n"
      " bar.red.or.pred q, %2, 256, p;\n selp.u32 %0, 1, 0, q;\n}\n"
      : "=r"(r)
      : "r"((uint32_t)v), "r"(id)
      : "memory");
  return r != 0;
}

__global__ void __launch_bounds__(512, 1)
    mlp_tc2_kernel(const __nv_bfloat16 *__restrict__ X, int n_atoms,
                   const __nv_bfloat16 *__restrict__ W1,
                   const float *__restrict__ b1,
                   const __nv_bfloat16 *__restrict__ W2,
                   const float *__restrict__ b2, const float *__restrict__ w3,
                   const float *__restrict__ b3, float *__restrict__ y,
                   __half *__restrict__ gout, int *err) {
  extern __shared__ unsigned char smem_raw[];
  const uint32_t raw = smem_addr(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  unsigned char *sp = smem_raw + (base - raw);
  float *sb1 = reinterpret_cast<float *>(sp + kOffVec2);
  float *sb2 = sb1 + kHid, *sw3 = sb2 + kHid;
  float *sy = reinterpret_cast<float *>(sp + kOffY2);
  uint32_t *slot_p = reinterpret_cast<uint32_t *>(sp + kOffBar2 + 16);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int s = warp >> 3;        // tile slot
  const int h = (warp >> 2) & 1;  // column half
  const int q = warp & 3;         // tensor-memory lane quarter
  const int r = 32 * q + lane;    // row of the tile
  const uint32_t bar = base + kOffBar2 + 8 * s;
  const int xo = kOffSlots + s * kSlotBytes;  // this slot's X block
  const int ao = xo + kBlk;                   // and activation blocks
  unsigned char *act = sp + ao;
  const int bar_id = 1 + s;
  const bool issuer = (tid & 255) == 0;

  for (int e = tid; e < kIn * kHid; e += blockDim.x) {
    const int c = e / kHid, hh = e % kHid;
    const __nv_bfloat16 v = W1[e];
    *reinterpret_cast<__nv_bfloat16 *>(sp + kOffW1T + bf16_at(hh, c)) = v;
    *reinterpret_cast<__nv_bfloat16 *>(sp + kOffW1 + (hh >> 6) * (32 * 128) +
                                       bf16_at(c, hh & 63)) = v;
  }
  for (int e = tid; e < kHid * kHid; e += blockDim.x) {
    const int i = e / kHid, o = e % kHid;
    const __nv_bfloat16 v = W2[e];
    *reinterpret_cast<__nv_bfloat16 *>(sp + kOffW2T + (i >> 6) * kBlk +
                                       bf16_at(o, i & 63)) = v;
    *reinterpret_cast<__nv_bfloat16 *>(sp + kOffW2 + (o >> 6) * kBlk +
                                       bf16_at(i, o & 63)) = v;
  }
  for (int e = tid; e < kHid; e += blockDim.x) {
    sb1[e] = b1[e];
    sb2[e] = b2[e];
    sw3[e] = w3[e];
  }
  if (tid == 0) {
    mbar_init(base + kOffBar2, 1);
    mbar_init(base + kOffBar2 + 8, 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncwarp();
  if (warp == 0) {
    asm volatile(
        "tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n"
        ::"r"(smem_addr(slot_p)), "r"(512)
        : "memory");
    asm volatile(
        "tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::
            : "memory");
  }
  fence_proxy_async();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem0 = *slot_p;
  const uint32_t tm = tmem0 + 256u * (uint32_t)s;
  const uint32_t lane_base = (uint32_t)(32 * q) << 16;
  const float bias3 = b3[0];
  const int n_tiles = (n_atoms + kRows - 1) / kRows;
  uint32_t phase = 0, n_done = 0;

  auto product = [&](uint32_t d, int a_off, int b_off, int b_blk, int n_k,
                     uint32_t idesc) {
    tc_fence_after();
    for (int k = 0; k < n_k; ++k) {
      const int kb = k >> 2, j = k & 3;
      const uint64_t da = sdesc(base + a_off + kb * kBlk + 32 * j);
      const uint64_t db = sdesc(base + b_off + kb * b_blk + 32 * j);
      mma_f16(d, da, db, idesc, k != 0);
    }
    mma_commit(bar);
  };
  auto wait_product = [&]() {
    const bool ok = mbar_wait(bar, phase & 1);
    ++phase;
    const bool bad = slot_sync_or(bar_id, !ok);
    tc_fence_after();
    return !bad;
  };
  auto to_product = [&]() {
    fence_proxy_async();
    tc_fence_before();
    slot_sync(bar_id);
  };

  for (int t = 2 * (int)blockIdx.x + s; t < n_tiles; t += 2 * (int)gridDim.x) {
    const int row = t * kRows + r;
    const bool have = row < n_atoms;
    {
      // half h stages chunks 2h, 2h + 1 of the X row
      const uint4 *xr = reinterpret_cast<const uint4 *>(X + (size_t)row * kIn);
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const int cc = 2 * h + c;
        const uint4 w = have ? xr[cc] : make_uint4(0u, 0u, 0u, 0u);
        *reinterpret_cast<uint4 *>(sp + xo + chunk_at(r, cc)) = w;
      }
    }
    to_product();
    if (issuer) product(tm, xo, kOffW1T, 0, kIn / 16, idesc_bf16(kRows, kHid));
    if (!wait_product()) break;

    // h1 = silu(z1 + b1), columns 64 h .. 64 h + 63
#pragma unroll 1
    for (int c0 = 64 * h; c0 < 64 * h + 64; c0 += 32) {
      float v[32];
      tmem_ld32(tm + lane_base + (uint32_t)c0, v);
#pragma unroll
      for (int k = 0; k < 32; ++k) v[k] = silu(v[k] + sb1[c0 + k]);
      store_row32(act, r, c0, v);
    }
    to_product();
    if (issuer)
      product(tm + 128, ao, kOffW2T, kBlk, kHid / 16, idesc_bf16(kRows, kHid));
    if (!wait_product()) break;

    // partial y and g2 = w3 * silu'(z2 + b2)
    float yp = h ? 0.f : bias3;
#pragma unroll 1
    for (int c0 = 64 * h; c0 < 64 * h + 64; c0 += 32) {
      float v[32];
      tmem_ld32(tm + 128 + lane_base + (uint32_t)c0, v);
#pragma unroll
      for (int k = 0; k < 32; ++k) {
        const float u = v[k] + sb2[c0 + k];
        yp = fmaf(silu(u), sw3[c0 + k], yp);
        v[k] = sw3[c0 + k] * dsilu(u);
      }
      store_row32(act, r, c0, v);
    }
    sy[(2 * s + h) * kRows + r] = yp;
    to_product();
    if (issuer)
      product(tm + 128, ao, kOffW2, kBlk, kHid / 16, idesc_bf16(kRows, kHid));
    if (!wait_product()) break;

    // g1 = gh1 * silu'(z1 + b1)
#pragma unroll 1
    for (int c0 = 64 * h; c0 < 64 * h + 64; c0 += 32) {
      float v[32], z[32];
      tmem_ld32(tm + 128 + lane_base + (uint32_t)c0, v);
      tmem_ld32(tm + lane_base + (uint32_t)c0, z);
#pragma unroll
      for (int k = 0; k < 32; ++k) v[k] *= dsilu(z[k] + sb1[c0 + k]);
      store_row32(act, r, c0, v);
    }
    to_product();
    if (issuer)
      product(tm, ao, kOffW1, 32 * 128, kHid / 16, idesc_bf16(kRows, kIn));
    if (!wait_product()) break;

    if (h == 0) {
      // gX -> FP16 row
      float v[32];
      tmem_ld32(tm + lane_base, v);
      if (have) {
        uint4 *gr = reinterpret_cast<uint4 *>(gout + (size_t)row * kIn);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          uint4 w;
          const __half2 h0 = __floats2half2_rn(v[8 * c + 0], v[8 * c + 1]);
          const __half2 h1 = __floats2half2_rn(v[8 * c + 2], v[8 * c + 3]);
          const __half2 h2 = __floats2half2_rn(v[8 * c + 4], v[8 * c + 5]);
          const __half2 h3 = __floats2half2_rn(v[8 * c + 6], v[8 * c + 7]);
          w.x = *reinterpret_cast<const uint32_t *>(&h0);
          w.y = *reinterpret_cast<const uint32_t *>(&h1);
          w.z = *reinterpret_cast<const uint32_t *>(&h2);
          w.w = *reinterpret_cast<const uint32_t *>(&h3);
          gr[c] = w;
        }
      }
    } else if (have) {
      y[row] = sy[(2 * s) * kRows + r] + sy[(2 * s + 1) * kRows + r];
    }
    ++n_done;
    // the next tile's products overwrite z1 / gX, X and the partial sums
    tc_fence_before();
    slot_sync(bar_id);
  }
  if (issuer && phase != 4u * n_done) {
    atomicCAS(err, 0, kErrAccumWait);
    // a product that timed out may still be writing tensor memory: one more
    // bounded wait for its commit before the columns are freed
    mbar_wait(bar, (phase - 1u) & 1u);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(
                     tmem0),
                 "r"(512)
                 : "memory");
  }
}

}  // namespace mlptc
}  // namespace pyiid
