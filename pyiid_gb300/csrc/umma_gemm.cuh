// 3xTF32 GEMM on the fifth-generation tensor cores (tcgen05), for the compat
// G(r) gradient: out[row][i] = sum_{k >= kmin} A[row][k] T[k][i], FP32 inputs,
// FP64 output (kernels/master_kernel.py:272-290 applies the F -> G map to
// each of the 3N rows of grad_fq).
//
// Accuracy: every operand x is split into x_hi = x with the low 13 mantissa
// bits cleared (exactly a TF32 value) and x_lo = x - x_hi (exact in FP32);
//   A T ~= A_lo T_hi + A_hi T_lo + A_hi T_hi
// with FP32 accumulation in tensor memory (A_lo T_lo and the bits of x_lo
// that a TF32 multiply ignores are below 2^-20 of each product).
//
// Data flow:
//   * pack kernels write A_hi, A_lo (per call) and T_hi, T_lo (once per T
//     matrix, transposed so that both operands are K-major) as blocks of
//     [rows][32 k] in the 128-byte swizzled order the tensor core's
//     shared-memory descriptors read; rows and k beyond the problem are
//     zero, so the main kernel has no edge cases but its stores;
//   * main kernel, persistent, one CTA per SM (the stages take 192 KB of
//     shared memory) walking 128 x BN output tiles: warp 0 lane 0 streams
//     the four tiles of each 32-wide k step into a ring of S stages with
//     bulk copies (cp.async.bulk, completion counted in bytes on an
//     mbarrier); warp 1 lane 0 issues 3 x 4 tcgen05.mma.kind::tf32 (M 128,
//     N BN, K 8) per k step into one of two 128 x BN FP32 accumulators in
//     tensor memory and frees the stage with tcgen05.commit; warps 2-5
//     read the other accumulator back with tcgen05.ld, stage it through
//     shared memory and store FP64 row segments.
// Every mbarrier wait is bounded: on time-out the kernel records an error
// code, waits (bounded) for the copies it started, frees its tensor memory
// and returns.
#pragma once

#include <cstdint>

namespace pyiid {
namespace umma {

constexpr int kBM = 128;        // rows of A per tile (tensor-memory lanes)
constexpr int kBK = 32;         // k per stage: 32 x 4 bytes = one swizzle row
constexpr int kTileA = kBM * kBK;  // floats per packed A tile
constexpr long long kSpinCycles = 2000000000LL;  // ~1 s at 2 GHz

// Position of element (r, k), k < 32, inside a packed [rows][32] block: rows
// of 128 bytes, 16-byte chunk c of row r stored at chunk c ^ (r mod 8) (the
// 128-byte swizzle; 8-row groups start on 1024-byte boundaries).
__host__ __device__ __forceinline__ int swizzled(int r, int k) {
  return r * kBK + ((((k >> 2) ^ (r & 7))) << 2) + (k & 3);
}

__device__ __forceinline__ void split_tf32(float x, float &hi, float &lo) {
  hi = __uint_as_float(__float_as_uint(x) & 0xffffe000u);
  lo = x - hi;
}

// Packed operand layout, for A (rows = rows of grad_fq) and for B = T^T
// (rows = r points): [k tile][rows_pad][32 k], k counted from kmin, each k
// tile a column of 8-row swizzle groups, so the rows of any tile of 128 or
// 256 rows at a given k tile are one contiguous block.

// A [n_rows][n_bins] (row stride n_bins) -> A_hi, A_lo.  One thread per
// packed element; a warp covers 32 consecutive k of one row.
__global__ void pack_a_kernel(const float *__restrict__ A, int n_rows,
                              int n_bins, int kmin, int rows_pad, int k_tiles,
                              float *__restrict__ a_hi,
                              float *__restrict__ a_lo) {
  const int kw = k_tiles * kBK;
  const long long total = (long long)rows_pad * kw;
  const size_t kstride = (size_t)rows_pad * kBK;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
       i < total; i += (long long)gridDim.x * blockDim.x) {
    const int row = (int)(i / kw), kk = (int)(i % kw);
    const int k = kmin + kk;
    const float x =
        (row < n_rows && k < n_bins) ? A[(size_t)row * n_bins + k] : 0.f;
    float hi, lo;
    split_tf32(x, hi, lo);
    const size_t dst = (size_t)(kk / kBK) * kstride + swizzled(row, kk % kBK);
    a_hi[dst] = hi;
    a_lo[dst] = lo;
  }
}

// T [n_bins][n_r] -> B_hi, B_lo (B = T^T, K-major).  One thread per element;
// a warp reads 32 consecutive r of one k; runs once per T matrix.
__global__ void pack_b_kernel(const float *__restrict__ T, int n_bins, int n_r,
                              int kmin, int rows_pad, int k_tiles,
                              float *__restrict__ b_hi,
                              float *__restrict__ b_lo) {
  const long long total = (long long)k_tiles * kBK * rows_pad;
  const size_t kstride = (size_t)rows_pad * kBK;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
       i < total; i += (long long)gridDim.x * blockDim.x) {
    const int kk = (int)(i / rows_pad), c = (int)(i % rows_pad);
    const int k = kmin + kk;
    const float x = (c < n_r && k < n_bins) ? T[(size_t)k * n_r + c] : 0.f;
    float hi, lo;
    split_tf32(x, hi, lo);
    const size_t dst = (size_t)(kk / kBK) * kstride + swizzled(c, kk % kBK);
    b_hi[dst] = hi;
    b_lo[dst] = lo;
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

// instruction descriptor, kind::tf32: D F32, A and B TF32, both K-major,
// N >> 3 at bit 17, M >> 4 at bit 24
__host__ __device__ constexpr uint32_t idesc_tf32(int m, int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a,
                                         uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(
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

// 16 consecutive FP32 columns of this thread's tensor-memory lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]),
        "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
        "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
        "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// error codes written to *err (0 = none)
enum : int { kErrFullWait = 1, kErrEmptyWait = 2, kErrAccumWait = 3 };

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
__device__ __forceinline__ double widen_f32(float x) {
  uint32_t u = __float_as_uint(x);
  const bool sub = ((u & 0x7f800000u) == 0u) && (u & 0x007fffffu);
  u = sub ? __float_as_uint(x * 16777216.0f) : u;
  const uint32_t e = (u >> 23) & 0xffu;
  const uint32_t bias =
      e == 0u ? 0u : (e == 255u ? 0x70000000u : 0x38000000u);
  const uint32_t hi =
      ((u & 0x80000000u) | (((u & 0x7fffffffu) >> 3) + bias)) -
      (sub ? (24u << 20) : 0u);
  return __hiloint2double((int)hi, (int)(u << 29));
}

template <int BN, int S>
struct PersistShape {
  static constexpr int kTileB = BN * kBK;
  static constexpr int kABytes = kTileA * 4;
  static constexpr int kBBytes = kTileB * 4;
  static constexpr int kStage = 2 * kABytes + 2 * kBBytes;
  // epilogue staging: 32 rows x 32 columns (FP32) per epilogue warp
  static constexpr int kStaging = 4 * 32 * kStagePitch * 4;
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
template <int BN, int S>
__global__ void __launch_bounds__(192, 1)
    tf32x3_gemm_persistent(const float *__restrict__ a_hi,
                           const float *__restrict__ a_lo,
                           const float *__restrict__ b_hi,
                           const float *__restrict__ b_lo, int k_tiles,
                           int a_rows_pad, int b_rows_pad, int m_tiles,
                           int n_tiles, int n_rows, int n_r,
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
      mbar_init(acc_empty(b), 4);  // one arrival per epilogue warp
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
  const size_t a_ks = (size_t)a_rows_pad * kBK, b_ks = (size_t)b_rows_pad * kBK;
  int issued = 0;

  if (tid == 0) {
    int g = 0;
    bool ok = true;
    for (int t = first; t < total && ok; t += stride) {
      const float *ah = a_hi + (size_t)row_tile(t) * kTileA;
      const float *al = a_lo + (size_t)row_tile(t) * kTileA;
      const float *bh = b_hi + (size_t)(t % n_tiles) * G::kTileB;
      const float *bl = b_lo + (size_t)(t % n_tiles) * G::kTileB;
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
    constexpr uint32_t idesc = idesc_tf32(kBM, BN);
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
        for (int j = 0; j < kBK / 8; ++j) {
          const uint64_t dah = sdesc(st + 32 * j);
          const uint64_t dal = sdesc(st + G::kABytes + 32 * j);
          const uint64_t dbh = sdesc(st + 2 * G::kABytes + 32 * j);
          const uint64_t dbl =
              sdesc(st + 2 * G::kABytes + G::kBBytes + 32 * j);
          mma_tf32(d, dal, dbh, idesc, (kt | j) != 0);
          mma_tf32(d, dah, dbl, idesc, 1u);
          mma_tf32(d, dah, dbh, idesc, 1u);
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
    const int q = warp & 3;
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
#pragma unroll 1
      for (int c = 0; c < BN; c += 32) {
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
            if (row < n_rows && col < n_r)
              *reinterpret_cast<double2 *>(out + (size_t)row * n_r + col) =
                  make_double2(widen_f32(stg[rr * kStagePitch + cc]),
                               widen_f32(stg[rr * kStagePitch + cc + 1]));
          }
        } else {
          const int col = col0 + c + lane;
#pragma unroll 4
          for (int rr = 0; rr < 32; ++rr) {
            const int row = row0 + rr;
            if (row < n_rows && col < n_r)
              out[(size_t)row * n_r + col] =
                  widen_f32(stg[rr * kStagePitch + lane]);
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
