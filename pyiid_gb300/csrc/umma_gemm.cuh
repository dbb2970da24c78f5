// GEMM on the fifth-generation tensor cores (tcgen05) with FP32-level
// accuracy, for the compat G(r) gradient: out[row][i] = sum_{k >= kmin}
// A[row][k] T[k][i], FP32 inputs, FP64 output (kernels/master_kernel.py:
// 272-290 applies the F -> G map to each of the 3N rows of grad_fq).
//
// Accuracy: each row of A (and T as a whole) is scaled by an exact power of
// two that puts its largest magnitude in [2^14, 2^15), and every scaled
// element is split into two FP16 halves, x = hi + lo (22 bits);
//   A T ~= A_hi T_hi + A_hi T_lo + A_lo T_hi
// as three tcgen05.mma.kind::f16 products with FP32 accumulation in tensor
// memory; the FP64 result is the accumulator times 2^-(e_row + e_T), applied
// exactly while widening.  Norm-wise error against FP64 ~1.2e-6 (a split
// into two TF32 halves, the same three products of kind::tf32, gave 2.7e-6
// and read twice the bytes per product).
//
// Data flow:
//   * pack kernels write A_hi, A_lo and the row exponents (per call) and
//     T_hi, T_lo (once per T matrix, transposed so that both operands are
//     K-major) as blocks of [rows][64 k] in the 128-byte swizzled order the
//     tensor core's shared-memory descriptors read; rows and k beyond the
//     problem are zero, so the main kernel has no edge cases but its
//     stores;
//   * main kernel, persistent, one CTA per SM (the stages take 192 KB of
//     shared memory) walking 128 x BN output tiles: warp 0 lane 0 streams
//     the four tiles of each 64-wide k step into a ring of S stages with
//     bulk copies (cp.async.bulk, completion counted in bytes on an
//     mbarrier); warp 1 lane 0 issues 3 x 4 tcgen05.mma.kind::f16 (M 128,
//     N BN, K 16) per k step into one of two 128 x BN FP32 accumulators in
//     tensor memory and frees the stage with tcgen05.commit; eight
//     epilogue warps read the other accumulator back with tcgen05.ld, stage
//     it through shared memory and store FP64 row segments.
// Every mbarrier wait is bounded: on time-out the kernel records an error
// code, waits (bounded) for the copies it started, frees its tensor memory
// and returns.
#pragma once

#include <cstdint>
#include <cuda_fp16.h>

namespace pyiid {
namespace umma {

constexpr int kBM = 128;        // rows of A per tile (tensor-memory lanes)
constexpr int kRowBytes = 128;  // one swizzle row of a packed operand
constexpr int kTileABytes = kBM * kRowBytes;
constexpr long long kSpinCycles = 2000000000LL;  // ~1 s at 2 GHz

// Packed operand layout, for A (rows = rows of grad_fq) and for B = T^T
// (rows = r points): [k tile][rows_pad][64 k] FP16, k counted from kmin,
// each k tile a column of 8-row swizzle groups, so the rows of any tile of
// 128 or 256 rows at a given k tile are one contiguous block.

// An operand row (a row of A, or all of T) is first scaled by an exact power
// of two 2^e that puts its largest magnitude in [2^14, 2^15) (FP16's range
// ends at 65504), then x 2^e = hi + lo with hi = fp16(x 2^e) and lo =
// fp16(x 2^e - hi) (the difference is exact in FP32): 22 bits of every
// element at least 2^-3 of the row's scale, and an absolute error below
// 2^-25 of it for the rest (FP16 subnormals).  A T ~= A_hi T_hi + A_hi T_lo +
// A_lo T_hi, and the FP64 result is the FP32 accumulator times
// 2^-(e_row + e_T), applied exactly in the widening.  A 128-byte swizzle
// row holds 64 k.
constexpr int kBK16 = 64;

// Position of element (r, k), k < 64, inside a packed [rows][64] block:
// rows of 128 bytes, 16-byte chunk c of row r stored at chunk c ^ (r mod 8)
// (the 128-byte swizzle; 8-row groups start on 1024-byte boundaries).
__host__ __device__ __forceinline__ int swizzled16(int r, int k) {
  return r * kBK16 + ((((k >> 3) ^ (r & 7))) << 3) + (k & 7);
}

// e such that amax 2^e lies in [2^14, 2^15); 0 for a zero or non-finite
// maximum; clamped to [-120, 120] (2^e stays a normal FP32 number; rows
// whose largest magnitude is below 2^-106 keep the clamped scale and lose
// low bits)
__host__ __device__ inline int fp16_scale_exp(float amax) {
  if (!(amax > 0.f) || !(amax <= 3.402823466e38f)) return 0;
  union {
    float f;
    uint32_t u;
  } c{amax};
  const int ex = (int)((c.u >> 23) & 0xffu) - 127;
  const int e = 14 - ex;
  return e < -120 ? -120 : (e > 120 ? 120 : e);
}

__device__ __forceinline__ float pow2f(int e) {  // e in [-126, 127]
  return __uint_as_float((uint32_t)(127 + e) << 23);
}

__device__ __forceinline__ void split_fp16(float xs, __half &hi, __half &lo) {
  hi = __float2half_rn(xs);
  lo = __float2half_rn(xs - __half2float(hi));
}

// A [n_rows][n_bins] -> A_hi, A_lo as [k tile][rows_pad][64 k] (FP16) and
// the scale exponent of every row.  One warp per row: the row's largest
// magnitude first, then the scaled split.
__global__ void pack_a_f16_kernel(const float *__restrict__ A, int n_rows,
                                  int n_bins, int kmin, int rows_pad,
                                  int k_tiles, __half *__restrict__ a_hi,
                                  __half *__restrict__ a_lo,
                                  int *__restrict__ row_exp) {
  const int lane = threadIdx.x & 31;
  const int nw = (int)((gridDim.x * blockDim.x) >> 5);
  const int kw = k_tiles * kBK16;
  const size_t kstride = (size_t)rows_pad * kBK16;
  for (int row = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
       row < rows_pad; row += nw) {
    const float *a = A + (size_t)row * n_bins;
    float amax = 0.f;
    if (row < n_rows)
      for (int k = kmin + lane; k < n_bins; k += 32)
        amax = fmaxf(amax, fabsf(a[k]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    const int e = fp16_scale_exp(amax);
    const float sc = pow2f(e);
    if (lane == 0) row_exp[row] = e;
    for (int kk = lane; kk < kw; kk += 32) {
      const int k = kmin + kk;
      const float x = (row < n_rows && k < n_bins) ? a[k] * sc : 0.f;
      __half h, l;
      split_fp16(x, h, l);
      const size_t dst =
          (size_t)(kk / kBK16) * kstride + swizzled16(row, kk % kBK16);
      a_hi[dst] = h;
      a_lo[dst] = l;
    }
  }
}

// T [n_bins][n_r] -> B_hi, B_lo (B = T^T, FP16, [k tile][rows_pad][64 k]),
// all scaled by 2^e_t.  One thread per element; runs once per T matrix.
__global__ void pack_b_f16_kernel(const float *__restrict__ T, int n_bins,
                                  int n_r, int kmin, int rows_pad,
                                  int k_tiles, int e_t,
                                  __half *__restrict__ b_hi,
                                  __half *__restrict__ b_lo) {
  const long long total = (long long)k_tiles * kBK16 * rows_pad;
  const size_t kstride = (size_t)rows_pad * kBK16;
  const float sc = pow2f(e_t);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
       i < total; i += (long long)gridDim.x * blockDim.x) {
    const int kk = (int)(i / rows_pad), c = (int)(i % rows_pad);
    const int k = kmin + kk;
    const float x =
        (c < n_r && k < n_bins) ? T[(size_t)k * n_r + c] * sc : 0.f;
    __half h, l;
    split_fp16(x, h, l);
    const size_t dst =
        (size_t)(kk / kBK16) * kstride + swizzled16(c, kk % kBK16);
    b_hi[dst] = h;
    b_lo[dst] = l;
  }
}

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar),
               "r"(count)
               : "memory");
}

// wait for the phase with the given parity; false after ~1 s
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  const long long t0 = clock64();
  while (true) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    if (clock64() - t0 > kSpinCycles) return false;
  }
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile(
      "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar),
      "r"(bytes)
      : "memory");
}

// global -> shared bulk copy (16-byte aligned addresses, size a multiple of
// 16), its bytes counted on the mbarrier
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src,
                                         uint32_t bytes, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1], %2, [%3];\n" ::"r"(dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}

// shared-memory matrix descriptor: K-major operand in 128-byte swizzled
// 8-row groups 1024 bytes apart (leading offset unused for this layout)
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) |
         ((uint64_t)(1024 >> 4) << 32) | ((uint64_t)1 << 46) |
         ((uint64_t)2 << 61);
}

// instruction descriptor, kind::f16 with FP16 A and B: D F32, both K-major
__host__ __device__ constexpr uint32_t idesc_f16(int m, int n) {
  return (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a,
                                        uint64_t b, uint32_t idesc,
                                        uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 "
      "[%0];\n" ::"r"(bar)
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(bar)
               : "memory");
}

// 32 consecutive FP32 columns of this thread's tensor-memory lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, "
      "%29, %30, %31}, [%32];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]),
        "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
        "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
        "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
        "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

constexpr int kStagePitch = 33;  // floats per staged row (conflict-free)

// FP32 -> FP64 on the integer pipes, exact for every non-NaN input (a NaN
// stays a NaN with its payload).  binary32 sign | 8-bit exponent | 23-bit
// fraction becomes binary64 sign | exponent + (1023 - 127) | fraction and 29
// zero bits; zero keeps only its sign; infinity and NaN take exponent 2047;
// a subnormal is first scaled by 2^24 (exact in FP32, then normal) and its
// binary64 exponent lowered by 24.  No branch and no conversion instruction:
// F2F.F64.F32 issues to the FP64 unit at about one result per clock per SM
// on this part, which made the 12 M conversions of a 3,000 x 4,000 output
// the limit of the whole GEMM (~20 us).
// x 2^-shift as binary64 (shift = 0: the plain widening); |shift| <= 300
// keeps every finite result a normal binary64
// (The shift is subtracted last, and only from finite nonzero values: with
// the shift folded into the selected bias the epilogue ran 35 % slower.)
__device__ __forceinline__ double widen_f32(float x, int shift = 0) {
  uint32_t u = __float_as_uint(x);
  const bool sub = ((u & 0x7f800000u) == 0u) && (u & 0x007fffffu);
  u = sub ? __float_as_uint(x * 16777216.0f) : u;
  const uint32_t e = (u >> 23) & 0xffu;
  const uint32_t bias =
      e == 0u ? 0u : (e == 255u ? 0x70000000u : 0x38000000u);
  uint32_t hi = ((u & 0x80000000u) | (((u & 0x7fffffffu) >> 3) + bias)) -
                (sub ? (24u << 20) : 0u);
  if (shift) hi -= (e - 1u < 254u) ? ((uint32_t)shift << 20) : 0u;
  return __hiloint2double((int)hi, (int)(u << 29));
}

// error codes written to *err (0 = none)
enum : int { kErrFullWait = 1, kErrEmptyWait = 2, kErrAccumWait = 3 };

// epilogue warps: two per tensor-memory lane quarter, each draining half
// of the accumulator's columns (four left the stores latency-bound)
constexpr int kEpiWarps = 8;
constexpr int kGemmThreads = 64 + 32 * kEpiWarps;

template <int BN, int S>
struct PersistShape {
  static constexpr int kABytes = kTileABytes;
  static constexpr int kBBytes = BN * kRowBytes;
  static constexpr int kStage = 2 * kABytes + 2 * kBBytes;
  // epilogue staging: 32 rows x 32 columns (FP32) per epilogue warp
  static constexpr int kStaging = kEpiWarps * 32 * kStagePitch * 4;
  // full[S], empty[S], acc_full[2], acc_empty[2], done
  static constexpr int kBars = 2 * S + 5;
  static constexpr int kSmem = 1024 + S * kStage + kStaging + 8 * kBars + 16;
  static constexpr int kCols = 2 * BN;  // two accumulators
  static_assert(kCols == 256 || kCols == 512, "tensor-memory columns");
  static_assert(kSmem <= 232448, "shared memory per CTA");
};

// Persistent form: one CTA per SM walks the output tiles t = blockIdx.x,
// blockIdx.x + gridDim.x, ... (row tile t / n_tiles, column tile
// t % n_tiles).  Warp 0 lane 0 streams stages, warp 1 lane 0 issues the
// MMAs into one of two accumulators (2 x BN tensor-memory columns), warps
// 2-5 drain the other accumulator (warp w reads lanes 32 (w mod 4) ..), so
// a tile's FP64 stores overlap the next tile's loads and products.
// The operands are the FP16 halves of pack_a_f16_kernel / pack_b_f16_kernel
// (byte addresses of the packed layouts); row r of the result is scaled by
// 2^-(row_exp[r] + e_t) in the widening.
template <int BN, int S>
__global__ void __launch_bounds__(kGemmThreads, 1)
    f16x2_gemm_persistent(const void *__restrict__ a_hi,
                           const void *__restrict__ a_lo,
                           const void *__restrict__ b_hi,
                           const void *__restrict__ b_lo, int k_tiles,
                           int a_rows_pad, int b_rows_pad, int m_tiles,
                           int n_tiles, int n_rows, int n_r,
                           const int *__restrict__ row_exp, int e_t,
                           double *__restrict__ out, int *err) {
  using G = PersistShape<BN, S>;
  extern __shared__ unsigned char smem_raw[];
  const uint32_t raw = smem_addr(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  unsigned char *sp = smem_raw + (base - raw);
  float *staging = reinterpret_cast<float *>(sp + S * G::kStage);
  const uint32_t bars = base + S * G::kStage + G::kStaging;
  uint32_t *words = reinterpret_cast<uint32_t *>(sp + S * G::kStage +
                                                 G::kStaging + 8 * G::kBars);
  // words[0] tensor-memory address, [1] error, [2] stages consumed
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  auto full = [&](int s) { return bars + 8 * s; };
  auto empty = [&](int s) { return bars + 8 * (S + s); };
  auto acc_full = [&](int b) { return bars + 8 * (2 * S + b); };
  auto acc_empty = [&](int b) { return bars + 8 * (2 * S + 2 + b); };
  const uint32_t done = bars + 8 * (2 * S + 4);
  const int total = m_tiles * n_tiles;
  const int first = (int)blockIdx.x, stride = (int)gridDim.x;
  auto row_tile = [&](int t) { return t / n_tiles; };

  if (tid == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(full(s), 1);
      mbar_init(empty(s), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(acc_full(b), 1);
      mbar_init(acc_empty(b), kEpiWarps);  // one arrival per epilogue warp
    }
    mbar_init(done, 1);
    words[1] = 0;
    words[2] = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncwarp();
  if (warp == 0) {
    asm volatile(
        "tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n"
        ::"r"(smem_addr(&words[0])), "r"(G::kCols)
        : "memory");
    asm volatile(
        "tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::
            : "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = words[0];
  // bytes from one k tile to the next (rows of 128 bytes)
  const size_t a_ks = (size_t)a_rows_pad * kRowBytes,
               b_ks = (size_t)b_rows_pad * kRowBytes;
  int issued = 0;

  if (tid == 0) {
    int g = 0;
    bool ok = true;
    for (int t = first; t < total && ok; t += stride) {
      const char *ah = static_cast<const char *>(a_hi) +
                       (size_t)row_tile(t) * G::kABytes;
      const char *al = static_cast<const char *>(a_lo) +
                       (size_t)row_tile(t) * G::kABytes;
      const char *bh = static_cast<const char *>(b_hi) +
                       (size_t)(t % n_tiles) * G::kBBytes;
      const char *bl = static_cast<const char *>(b_lo) +
                       (size_t)(t % n_tiles) * G::kBBytes;
      for (int kt = 0; kt < k_tiles; ++kt, ++g) {
        const int s = g % S, use = g / S;
        if (use > 0 && !mbar_wait(empty(s), (use - 1) & 1)) {
          atomicCAS(&words[1], 0u, (unsigned)kErrEmptyWait);
          ok = false;
          break;
        }
        const uint32_t st = base + s * G::kStage;
        mbar_expect_tx(full(s), G::kStage);
        bulk_g2s(st, ah + kt * a_ks, G::kABytes, full(s));
        bulk_g2s(st + G::kABytes, al + kt * a_ks, G::kABytes, full(s));
        bulk_g2s(st + 2 * G::kABytes, bh + kt * b_ks, G::kBBytes, full(s));
        bulk_g2s(st + 2 * G::kABytes + G::kBBytes, bl + kt * b_ks,
                 G::kBBytes, full(s));
        issued = g + 1;
      }
    }
  } else if (tid == 32) {
    constexpr uint32_t idesc = idesc_f16(kBM, BN);
    int g = 0, li = 0;
    bool ok = true;
    for (int t = first; t < total && ok; t += stride, ++li) {
      const int b = li & 1, ub = li >> 1;
      if (ub > 0 && !mbar_wait(acc_empty(b), (ub - 1) & 1)) {
        atomicCAS(&words[1], 0u, (unsigned)kErrAccumWait);
        break;
      }
      tc_fence_after();
      const uint32_t d = tmem + (uint32_t)(b * BN);
      for (int kt = 0; kt < k_tiles; ++kt, ++g) {
        const int s = g % S;
        if (!mbar_wait(full(s), (g / S) & 1)) {
          atomicCAS(&words[1], 0u, (unsigned)kErrFullWait);
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t st = base + s * G::kStage;
#pragma unroll
        for (int j = 0; j < kRowBytes / 32; ++j) {  // 4 MMAs of K 16 (32 bytes)
          const uint64_t dah = sdesc(st + 32 * j);
          const uint64_t dal = sdesc(st + G::kABytes + 32 * j);
          const uint64_t dbh = sdesc(st + 2 * G::kABytes + 32 * j);
          const uint64_t dbl =
              sdesc(st + 2 * G::kABytes + G::kBBytes + 32 * j);
          mma_f16(d, dal, dbh, idesc, (kt | j) != 0);
          mma_f16(d, dah, dbl, idesc, 1u);
          mma_f16(d, dah, dbh, idesc, 1u);
        }
        mma_commit(empty(s));
      }
      if (ok) mma_commit(acc_full(b));
    }
    words[2] = g;
    mma_commit(done);
  } else if (warp >= 2) {
    // epilogue: warp w owns accumulator lanes (rows) 32 (w mod 4) .. + 31;
    // each 32 x 32 block goes through shared memory so that the FP64
    // stores are row segments of 256 bytes (two rows per instruction)
    const int q = warp & 3;  // lane quarter (tcgen05.ld: warp w, lanes 32 (w mod 4) ..)
    const int half = (warp - 2) / 4;  // which half of the columns
    float *stg = staging + (warp - 2) * 32 * kStagePitch;
    const bool pairs =
        (n_r % 2) == 0 && (reinterpret_cast<uintptr_t>(out) & 15) == 0;
    int li = 0;
    for (int t = first; t < total; t += stride, ++li) {
      const int b = li & 1, ub = li >> 1;
      // the warp leaves together (the loads below are warp-collective)
      if (!__all_sync(0xffffffffu, mbar_wait(acc_full(b), ub & 1))) {
        if (lane == 0) atomicCAS(&words[1], 0u, (unsigned)kErrAccumWait);
        break;
      }
      tc_fence_after();
      const int row0 = row_tile(t) * kBM + q * 32;
      const int col0 = (t % n_tiles) * BN;
      // scale exponent of this lane's row (rows of the padded operand, so
      // always in range); other lanes' rows by shuffle
      const int my_shift = row_exp[row0 + lane] + e_t;
#pragma unroll 1
      for (int c = half * (BN / 2); c < (half + 1) * (BN / 2); c += 32) {
        __syncwarp();  // staging free, warp converged for tcgen05.ld
        float v[32];
        tmem_ld32(tmem + (uint32_t)(b * BN) + ((uint32_t)(q * 32) << 16) +
                      (uint32_t)c,
                  v);
#pragma unroll
        for (int j = 0; j < 32; ++j) stg[lane * kStagePitch + j] = v[j];
        __syncwarp();
        if (pairs) {
          const int cc = 2 * (lane & 15), col = col0 + c + cc;
#pragma unroll 4
          for (int i = 0; i < 16; ++i) {
            const int rr = 2 * i + (lane >> 4), row = row0 + rr;
            const int sh = __shfl_sync(0xffffffffu, my_shift, rr);
            if (row < n_rows && col < n_r)
              *reinterpret_cast<double2 *>(out + (size_t)row * n_r + col) =
                  make_double2(widen_f32(stg[rr * kStagePitch + cc], sh),
                               widen_f32(stg[rr * kStagePitch + cc + 1], sh));
          }
        } else {
          const int col = col0 + c + lane;
#pragma unroll 4
          for (int rr = 0; rr < 32; ++rr) {
            const int row = row0 + rr;
            const int sh = __shfl_sync(0xffffffffu, my_shift, rr);
            if (row < n_rows && col < n_r)
              out[(size_t)row * n_r + col] =
                  widen_f32(stg[rr * kStagePitch + lane], sh);
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(acc_empty(b));
    }
  }
  __syncthreads();
  if (tid == 0) {
    // every MMA this CTA issued has completed once `done` fires; copies
    // started but never consumed (only after a time-out) land before the
    // shared memory is released
    if (!mbar_wait(done, 0)) atomicCAS(&words[1], 0u, (unsigned)kErrAccumWait);
    for (int g = (int)words[2]; g < issued; ++g)
      mbar_wait(full(g % S), (g / S) & 1);
    if (words[1]) atomicCAS(err, 0, (int)words[1]);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(
                     tmem),
                 "r"(G::kCols)
                 : "memory");
  }
}

}  // namespace umma
}  // namespace pyiid
