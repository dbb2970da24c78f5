// surrogate_kernels.cuh -- the learned first stage of delayed acceptance.
//
// Per-atom radial-basis descriptors and a small MLP whose summed per-atom
// outputs estimate a configuration's Rw.  The MLP layers are BF16 GEMMs on
// the tensor cores (mma.sync m16n8k16, FP32 accumulate); the descriptors and
// activations are plain FP32 kernels.  Shapes are small (32 -> 128 -> 128 ->
// 1 per atom), so the GEMM favours simplicity: 64 x 64 CTA tiles staged in
// shared memory, one K step of 16 per iteration.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

namespace pyiid {

// ------------------------------------------------------------- descriptors
// feat[a][c] = sum_{b != a, same configuration} exp(-(r - mu_c)^2 / (2 s^2))
//              * fc(r),   mu_c = c * rc / (C - 1),  fc(r) = (1 + cos(pi r/rc))/2
// for r < rc (0 beyond).  One warp per atom a; lane l owns centres l, l+32
// (C <= 64), every lane walks all b of the configuration (uniform branches,
// broadcast loads), so no atomics are needed.  Written as BF16 (the MLP
// input) and optionally FP32.
__global__ void rbf_features_kernel(const float *__restrict__ pos,
                                    const int *__restrict__ atom_cfg,
                                    const int *__restrict__ offsets,
                                    int n_atoms, int n_centres, float rc,
                                    float sigma, __nv_bfloat16 *__restrict__ fb,
                                    float *__restrict__ ff) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int a = blockIdx.x * (blockDim.x >> 5) + warp;
  if (a >= n_atoms) return;
  const int cfg = atom_cfg[a];
  const int b0 = offsets[cfg], b1 = offsets[cfg + 1];
  const float ax = pos[3 * a], ay = pos[3 * a + 1], az = pos[3 * a + 2];
  const float step = rc / (float)(n_centres - 1);
  const float inv2s2 = 0.5f / (sigma * sigma);
  const float mu0 = lane * step, mu1 = (lane + 32) * step;
  const float rc2 = rc * rc;
  float acc0 = 0.f, acc1 = 0.f;
  for (int b = b0; b < b1; ++b) {
    const float dx = pos[3 * b] - ax, dy = pos[3 * b + 1] - ay,
                dz = pos[3 * b + 2] - az;
    const float r2 = dx * dx + dy * dy + dz * dz;
    if (b == a || r2 >= rc2) continue;
    const float r = sqrtf(r2);
    const float fc = 0.5f * (1.f + cospif(r / rc));
    const float d0 = r - mu0, d1 = r - mu1;
    acc0 = fmaf(fc, __expf(-d0 * d0 * inv2s2), acc0);
    acc1 = fmaf(fc, __expf(-d1 * d1 * inv2s2), acc1);
  }
  if (lane < n_centres) {
    fb[(size_t)a * n_centres + lane] = __float2bfloat16_rn(acc0);
    if (ff) ff[(size_t)a * n_centres + lane] = acc0;
  }
  if (lane + 32 < n_centres) {
    fb[(size_t)a * n_centres + lane + 32] = __float2bfloat16_rn(acc1);
    if (ff) ff[(size_t)a * n_centres + lane + 32] = acc1;
  }
}

// ------------------------------------------------------------------- GEMM
// C[M][N] (+)= op(A) op(B), BF16 inputs, FP32 accumulate and output.
//   TA = false: A is [M][K] row-major (lda); TA = true: A is stored [K][M].
//   TB = false: B is [K][N] row-major (ldb); TB = true: B is stored [N][K].
// CTA tile 64 x 64, 4 warps each owning a 32 x 32 sub-tile (2 x 4 mma tiles
// of 16 x 8), K stepped by 16 through shared memory.  Out-of-range elements
// are loaded as zero and never stored.
//
// mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 fragments (per lane,
// g = lane / 4, q = lane % 4):
//   A: a0 = (g, 2q..2q+1), a1 = (g+8, 2q..), a2 = (g, 2q+8..), a3 = (g+8, 2q+8..)
//   B: b0 = (k 2q..2q+1, n g), b1 = (k 2q+8.., n g)
//   C: c0 = (g, 2q), c1 = (g, 2q+1), c2 = (g+8, 2q), c3 = (g+8, 2q+1)
__device__ __forceinline__ unsigned pack_bf16(__nv_bfloat16 lo,
                                              __nv_bfloat16 hi) {
  const unsigned short l = __bfloat16_as_ushort(lo);
  const unsigned short h = __bfloat16_as_ushort(hi);
  return (unsigned)l | ((unsigned)h << 16);
}

__device__ __forceinline__ void mma_bf16_16816(float (&c)[4], const unsigned (&a)[4],
                                               const unsigned (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

template <bool TA, bool TB>
__global__ void __launch_bounds__(128)
    gemm_bf16_kernel(const __nv_bfloat16 *__restrict__ A, int lda,
                     const __nv_bfloat16 *__restrict__ B, int ldb,
                     float *__restrict__ C, int ldc, int M, int N, int K,
                     int accumulate) {
  __shared__ __nv_bfloat16 sA[64][16 + 8];  // [m][k]
  __shared__ __nv_bfloat16 sB[64][16 + 8];  // [n][k]
  const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int g = lane >> 2, q = lane & 3;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[i][j][e] = 0.f;
  const __nv_bfloat16 z = __float2bfloat16_rn(0.f);
  for (int k0 = 0; k0 < K; k0 += 16) {
    for (int e = tid; e < 64 * 16; e += 128) {
      const int r = e / 16, kk = e % 16;
      const int gm = m0 + r, gk = k0 + kk;
      __nv_bfloat16 v = z;
      if (gm < M && gk < K)
        v = TA ? A[(size_t)gk * lda + gm] : A[(size_t)gm * lda + gk];
      sA[r][kk] = v;
      const int gn = n0 + r;
      __nv_bfloat16 w = z;
      if (gn < N && gk < K)
        w = TB ? B[(size_t)gn * ldb + gk] : B[(size_t)gk * ldb + gn];
      sB[r][kk] = w;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const int r = wm + i * 16;
      unsigned af[4];
      af[0] = pack_bf16(sA[r + g][2 * q], sA[r + g][2 * q + 1]);
      af[1] = pack_bf16(sA[r + g + 8][2 * q], sA[r + g + 8][2 * q + 1]);
      af[2] = pack_bf16(sA[r + g][2 * q + 8], sA[r + g][2 * q + 9]);
      af[3] = pack_bf16(sA[r + g + 8][2 * q + 8], sA[r + g + 8][2 * q + 9]);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int cn = wn + j * 8;
        unsigned bf[2];
        bf[0] = pack_bf16(sB[cn + g][2 * q], sB[cn + g][2 * q + 1]);
        bf[1] = pack_bf16(sB[cn + g][2 * q + 8], sB[cn + g][2 * q + 9]);
        mma_bf16_16816(acc[i][j], af, bf);
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int gm = m0 + wm + i * 16 + g + (e >= 2 ? 8 : 0);
        const int gn = n0 + wn + j * 8 + 2 * q + (e & 1);
        if (gm < M && gn < N) {
          float *p = C + (size_t)gm * ldc + gn;
          *p = accumulate ? *p + acc[i][j][e] : acc[i][j][e];
        }
      }
}

// --------------------------------------------------------- elementwise ops
// h = silu(z + bias) for z [rows][n] (FP32 in place), also as BF16.
//   silu(x) = x / (1 + e^-x)
__global__ void bias_silu_kernel(float *__restrict__ z,
                                 const float *__restrict__ bias, int rows,
                                 int n, __nv_bfloat16 *__restrict__ hb,
                                 float *__restrict__ pre) {
  const size_t total = (size_t)rows * n;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const float x = z[i] + bias[i % n];
    if (pre) pre[i] = x;
    const float h = x / (1.f + __expf(-x));
    z[i] = h;
    hb[i] = __float2bfloat16_rn(h);
  }
}

// dz = dh * silu'(pre),  silu'(x) = s (1 + x (1 - s)),  s = 1 / (1 + e^-x);
// written as BF16 for the next GEMMs and FP32.
__global__ void silu_backward_kernel(const float *__restrict__ dh,
                                     const float *__restrict__ pre,
                                     size_t total,
                                     __nv_bfloat16 *__restrict__ dzb,
                                     float *__restrict__ dz) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const float x = pre[i];
    const float s = 1.f / (1.f + __expf(-x));
    const float v = dh[i] * s * (1.f + x * (1.f - s));
    dz[i] = v;
    dzb[i] = __float2bfloat16_rn(v);
  }
}

// Output layer and per-configuration sum: y[a] = h2[a] . w3 + b3,
// e[cfg] = sum_a y[a] (FP64).  One warp per atom; per-configuration sums
// are reduced by reduce_by_config_kernel.
__global__ void head_kernel(const float *__restrict__ h2,
                            const float *__restrict__ w3, const float *b3,
                            int rows, int n, float *__restrict__ y) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= rows) return;
  float s = 0.f;
  for (int i = lane; i < n; i += 32) s = fmaf(h2[(size_t)warp * n + i], w3[i], s);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) y[warp] = s + b3[0];
}

__global__ void reduce_by_config_kernel(const float *__restrict__ y,
                                        const int *__restrict__ offsets,
                                        int n_configs,
                                        double *__restrict__ e) {
  const int c = blockIdx.x;
  if (c >= n_configs) return;
  __shared__ double sm[256];
  double s = 0.0;
  for (int a = offsets[c] + threadIdx.x; a < offsets[c + 1]; a += blockDim.x)
    s += (double)y[a];
  sm[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) e[c] = sm[0];
}

// Head backward: given dL/de[cfg] (FP64), dy[a] = dL/de[cfg(a)];
//   dh2[a][i] = dy[a] w3[i]  (FP32 and BF16), dw3[i] = sum_a dy[a] h2[a][i],
//   db3 = sum_a dy[a].
__global__ void head_backward_kernel(const double *__restrict__ de,
                                     const int *__restrict__ atom_cfg,
                                     const float *__restrict__ h2,
                                     const float *__restrict__ w3, int rows,
                                     int n, float *__restrict__ dh2,
                                     __nv_bfloat16 *__restrict__ dh2b) {
  const size_t total = (size_t)rows * n;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int a = (int)(i / n), j = (int)(i % n);
    const float v = (float)de[atom_cfg[a]] * w3[j];
    dh2[i] = v;
    dh2b[i] = __float2bfloat16_rn(v);
  }
}

// Column sums over rows: out[j] = sum_a M[a][j] * (scale ? scale[a] : 1)
// (bias gradients; dw3 with scale = dy per row).  One block per column.
__global__ void column_sum_kernel(const float *__restrict__ Mx, int rows,
                                  int n, const double *__restrict__ de,
                                  const int *__restrict__ atom_cfg,
                                  float *__restrict__ out) {
  const int j = blockIdx.x;
  __shared__ double sm[256];
  double s = 0.0;
  for (int a = threadIdx.x; a < rows; a += blockDim.x) {
    const double w = de ? de[atom_cfg[a]] : 1.0;
    s += w * (Mx ? (double)Mx[(size_t)a * n + j] : 1.0);
  }
  sm[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[j] = (float)sm[0];
}

// ------------------------------------------------ neighbour-list variants
// Neighbour lists: for every atom a, the atoms b != a of its configuration
// with |x_a - x_b|^2 < r_list2, in increasing b.  count[a] is the number
// found; entries beyond max_nb are not stored, so count[a] > max_nb flags an
// overflow.  One warp per atom: lanes test b = b0 + lane + 32 t and a ballot
// compacts the hits in b order.
__global__ void neighbor_list_kernel(const float *__restrict__ pos,
                                     const int *__restrict__ atom_cfg,
                                     const int *__restrict__ offsets,
                                     int n_atoms, float r_list2, int max_nb,
                                     int *__restrict__ nbr,
                                     int *__restrict__ count) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int a = blockIdx.x * (blockDim.x >> 5) + warp;
  if (a >= n_atoms) return;  // whole warps leave together
  const int cfg = atom_cfg[a];
  const int b0 = offsets[cfg], b1 = offsets[cfg + 1];
  const float ax = pos[3 * a], ay = pos[3 * a + 1], az = pos[3 * a + 2];
  int n = 0;
  for (int base = b0; base < b1; base += 32) {
    const int b = base + lane;
    bool hit = false;
    if (b < b1 && b != a) {
      const float dx = pos[3 * b] - ax, dy = pos[3 * b + 1] - ay,
                  dz = pos[3 * b + 2] - az;
      hit = dx * dx + dy * dy + dz * dz < r_list2;
    }
    const unsigned m = __ballot_sync(0xffffffffu, hit);
    if (hit) {
      const int slot = n + __popc(m & ((1u << lane) - 1u));
      if (slot < max_nb) nbr[(size_t)a * max_nb + slot] = b;
    }
    n += __popc(m);
  }
  if (lane == 0) count[a] = n;
}

// Warp reduce-scatter of 32 per-lane vectors acc[0..31]: afterwards lane l
// holds sum over lanes of acc[l] in acc[0].  Five butterfly steps; at offset
// o a lane keeps the half of its live entries selected by bit o of its index
// and adds the partner's copy of that half (31 shuffles instead of 32 x 5).
__device__ __forceinline__ float warp_reduce_scatter32(float (&acc)[32]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int i = 0; i < o; ++i) {
      const float send = up ? acc[i] : acc[i + o];
      const float keep = up ? acc[i + o] : acc[i];
      acc[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
    }
  }
  return acc[0];
}

// rbf_features_kernel over a neighbour list: one warp per atom, lane l takes
// the neighbours l, l + 32, ... (distance, cutoff and the C Gaussians per
// pair computed once), then a reduce-scatter gives lane c the sum of centre
// c (and c + 32 in a second pass when C > 32).  The same terms as the
// all-pairs kernel, summed in another order.
// 2^x by the hardware's base-2 exponential (ex2.approx, relative error of
// order 2^-22 over the range used here)
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__global__ void rbf_features_nl_kernel(const float *__restrict__ pos,
                                       const int *__restrict__ nbr,
                                       const int *__restrict__ count,
                                       int max_nb, int n_atoms, int n_centres,
                                       float rc, float sigma,
                                       __nv_bfloat16 *__restrict__ fb,
                                       float *__restrict__ ff) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int a = blockIdx.x * (blockDim.x >> 5) + warp;
  if (a >= n_atoms) return;
  const int n = min(count[a], max_nb);
  const int *nb = nbr + (size_t)a * max_nb;
  const float ax = pos[3 * a], ay = pos[3 * a + 1], az = pos[3 * a + 2];
  const float step = rc / (float)(n_centres - 1);
  // exp(-d^2 / (2 s^2)) = 2^(-c2 d^2), c2 = log2(e) / (2 s^2)
  const float c2 = 0.5f / (sigma * sigma) * 1.4426950408889634f;
  const float rc2 = rc * rc;
  for (int c0 = 0; c0 < n_centres; c0 += 32) {
    float acc[32];
#pragma unroll
    for (int c = 0; c < 32; ++c) acc[c] = 0.f;
    // the next neighbour's position is gathered while this one's Gaussians
    // are summed (the gathers were the kernel's top stall)
    float bx = 0.f, by = 0.f, bz = 0.f;
    if (lane < n) {
      const int b = nb[lane];
      bx = pos[3 * b];
      by = pos[3 * b + 1];
      bz = pos[3 * b + 2];
    }
    for (int i = lane; i < n; i += 32) {
      const float dx = bx - ax, dy = by - ay, dz = bz - az;
      if (i + 32 < n) {
        const int b = nb[i + 32];
        bx = pos[3 * b];
        by = pos[3 * b + 1];
        bz = pos[3 * b + 2];
      }
      const float r2 = dx * dx + dy * dy + dz * dz;
      if (r2 >= rc2) continue;
      const float r = sqrtf(r2);
      const float fc = 0.5f * (1.f + cospif(r / rc));
#pragma unroll
      for (int c = 0; c < 32; ++c) {
        const float d = r - (float)(c0 + c) * step;
        acc[c] = fmaf(fc, ex2_approx(-c2 * (d * d)), acc[c]);
      }
    }
    const float v = warp_reduce_scatter32(acc);
    const int c = c0 + lane;
    if (c < n_centres) {
      fb[(size_t)a * n_centres + c] = __float2bfloat16_rn(v);
      if (ff) ff[(size_t)a * n_centres + c] = v;
    }
  }
}

// out[a][j] = v[j] for every row a (FP32 and BF16): dE/dh2 when
// E = sum_a y_a.
__global__ void broadcast_rows_kernel(const float *__restrict__ v, int rows,
                                      int n, float *__restrict__ out,
                                      __nv_bfloat16 *__restrict__ outb) {
  const size_t total = (size_t)rows * n;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const float x = v[i % n];
    out[i] = x;
    outb[i] = __float2bfloat16_rn(x);
  }
}

// Forces of the surrogate energy E = sum_a y_a from g[a][c] = dE/dfeat[a][c]:
//   dE/dx_a = sum_{b in list(a), r_ab < rc} sum_c (g[a][c] + g[b][c])
//             phi_c'(r_ab) (x_a - x_b) / r_ab,
//   phi_c(r) = exp(-(r - mu_c)^2 / (2 s^2)) fc(r),
//   phi_c'(r) = exp(-(r - mu_c)^2 / (2 s^2)) (fc'(r) - fc(r) (r - mu_c)/s^2),
//   fc'(r) = -(pi / (2 rc)) sin(pi r / rc),
// (the descriptor of b holds the pair too), forces[a] = -scale dE/dx_a.  One
// warp per atom; lane l takes the neighbours l, l + 32, ... and loops over
// the centres with g[a] in registers and g[b] read 16 bytes at a time
// (FP32 or FP16 rows); the x, y, z sums are reduced over the warp once per
// atom.  n_centres % 4 == 0 (FP32) or % 8 == 0 (FP16), n_centres <= 64.
__device__ __forceinline__ void load_g8(const float *p, float (&v)[8]) {
  const float4 a = reinterpret_cast<const float4 *>(p)[0];
  const float4 b = reinterpret_cast<const float4 *>(p)[1];
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
  v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}
__device__ __forceinline__ void load_g8(const __half *p, float (&v)[8]) {
  const uint4 u = *reinterpret_cast<const uint4 *>(p);
  const unsigned w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float2 f = __half22float2(*reinterpret_cast<const __half2 *>(&w[i]));
    v[2 * i] = f.x;
    v[2 * i + 1] = f.y;
  }
}

template <typename GT>
__global__ void rbf_forces_nl_kernel(const float *__restrict__ pos,
                                     const int *__restrict__ nbr,
                                     const int *__restrict__ count,
                                     int max_nb, int n_atoms, int n_centres,
                                     float rc, float sigma,
                                     const GT *__restrict__ g, float scale,
                                     float *__restrict__ forces) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int a = blockIdx.x * (blockDim.x >> 5) + warp;
  if (a >= n_atoms) return;
  const int n = min(count[a], max_nb);
  const int *nb = nbr + (size_t)a * max_nb;
  const float ax = pos[3 * a], ay = pos[3 * a + 1], az = pos[3 * a + 2];
  const float step = rc / (float)(n_centres - 1);
  const float inv_s2 = 1.f / (sigma * sigma);
  // exp(-d^2 / (2 s^2)) = 2^(-c2 d^2), c2 = log2(e) / (2 s^2): the argument
  // in base 2 directly (one multiply fewer per term than exp)
  const float c2 = 0.5f * inv_s2 * 1.4426950408889634f;
  const float rc2 = rc * rc;
  const float kfc = -0.5f * 3.14159265358979f / rc;
  const GT *ga = g + (size_t)a * n_centres;
  // centres more than 6.5 sigma from r add less than exp(-21) of the
  // largest term: only the blocks of 8 centres within that window are
  // summed (about 21 of 32 terms when sigma is the centre spacing)
  const int win = (int)ceilf(6.5f * sigma / step);
  const int nq = n_centres / 8;
  float fx = 0.f, fy = 0.f, fz = 0.f;
  for (int i = lane; i < n; i += 32) {
    const int b = nb[i];
    const float dx = ax - pos[3 * b], dy = ay - pos[3 * b + 1],
                dz = az - pos[3 * b + 2];
    const float r2 = dx * dx + dy * dy + dz * dz;
    if (r2 >= rc2) continue;
    const float r = sqrtf(r2);
    float sn, cs;
    sincospif(r / rc, &sn, &cs);
    const float fc = 0.5f * (1.f + cs), dfc = kfc * sn;
    const GT *gb = g + (size_t)b * n_centres;
    const int k0 = __float2int_rn(r / step);
    const int q_lo = max(0, k0 - win) / 8;
    const int q_hi = min(nq - 1, max(0, k0 + win) / 8);
    float s = 0.f;
    for (int q = q_lo; q <= q_hi; ++q) {
      float u[8], w[8];
      load_g8(ga + 8 * q, u);
      load_g8(gb + 8 * q, w);
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        const float d = r - (float)(8 * q + e) * step;
        s = fmaf(u[e] + w[e], ex2_approx(-c2 * (d * d)) *
                                  (dfc - fc * d * inv_s2), s);
      }
    }
    s = s / r;
    fx = fmaf(s, dx, fx);
    fy = fmaf(s, dy, fy);
    fz = fmaf(s, dz, fz);
  }
  for (int o = 16; o > 0; o >>= 1) {
    fx += __shfl_xor_sync(0xffffffffu, fx, o);
    fy += __shfl_xor_sync(0xffffffffu, fy, o);
    fz += __shfl_xor_sync(0xffffffffu, fz, o);
  }
  if (lane == 0) {
    forces[3 * (size_t)a] = -scale * fx;
    forces[3 * (size_t)a + 1] = -scale * fy;
    forces[3 * (size_t)a + 2] = -scale * fz;
  }
}

// ------------------------------------------- fused MLP for the 32-128-128 net
// Forward and descriptor gradient of the per-atom MLP for n_in = 32,
// n_hidden = 128 in one kernel:
//   z1 = X W1 + b1, h1 = silu(z1), z2 = h1 W2 + b2, y = silu(z2) . w3 + b3,
//   g = dE/dX = ((w3 * silu'(z2)) W2^T * silu'(z1)) W1^T   (E = sum_a y_a).
// A warp owns 16 atoms; every product is an mma.sync m16n8k16 (BF16 in,
// FP32 accumulate) and the activations never leave registers: the FP32
// accumulator fragments of one layer, rounded to BF16 and paired, are
// exactly the A fragments of the next (C frag (g, 2q..2q+1) / (g+8, ..)
// of column tiles 2t and 2t+1 = A frag of k-tile t).  z1 is recomputed tile
// by tile in the backward pass instead of being kept.  The four weight
// layouts the B fragments need (consecutive k in one 32-bit word) are staged
// once per CTA in shared memory with padded rows (conflict-free loads); CTAs
// stay resident and loop over atom blocks (any multiple of 32 threads per
// CTA; the warps share the staged weights).  y is written per atom (summed
// per configuration by reduce_by_config_kernel) and g as FP16 [n][32] (the
// force kernel gathers one row per neighbour: half the bytes of FP32).
constexpr int kFC = 32, kFH = 128;
constexpr int kLd1 = kFC + 8;   // rows of 32 (+8 pad) bf16: W1T [h][c]
constexpr int kLd2 = kFH + 8;   // rows of 128 (+8 pad): W2T, W2, W1
struct FusedMlpSmem {
  __nv_bfloat16 w1t[kFH * kLd1];  // B of layer 1:  [h][c]
  __nv_bfloat16 w2t[kFH * kLd2];  // B of layer 2:  [o][i]
  __nv_bfloat16 w2[kFH * kLd2];   // B of dh1:      [i][o]
  __nv_bfloat16 w1[kFC * kLd2];   // B of g:        [c][h]
  float b1[kFH], b2[kFH], w3[kFH];
};

__device__ __forceinline__ unsigned pack2f(float lo, float hi) {
  return pack_bf16(__float2bfloat16_rn(lo), __float2bfloat16_rn(hi));
}
__device__ __forceinline__ float silu_f(float x) {
  return x / (1.f + __expf(-x));
}
__device__ __forceinline__ float dsilu_f(float x) {
  const float s = 1.f / (1.f + __expf(-x));
  return s * (1.f + x * (1.f - s));
}
__device__ __forceinline__ unsigned ld_u32(const __nv_bfloat16 *p) {
  return *reinterpret_cast<const unsigned *>(p);
}

__global__ void __launch_bounds__(256, 2)
    mlp_fused_kernel(const __nv_bfloat16 *__restrict__ X, int n_atoms,
                     const __nv_bfloat16 *__restrict__ W1,
                     const float *__restrict__ b1,
                     const __nv_bfloat16 *__restrict__ W2,
                     const float *__restrict__ b2,
                     const float *__restrict__ w3, const float *__restrict__ b3,
                     float *__restrict__ y, __half *__restrict__ gout) {
  extern __shared__ __align__(16) unsigned char fused_smem[];
  FusedMlpSmem &S = *reinterpret_cast<FusedMlpSmem *>(fused_smem);
  const int tid = threadIdx.x;
  // stage the weights: W1 [c][h], W2 [i][o] row-major in global memory
  for (int e = tid; e < kFC * kFH; e += blockDim.x) {
    const int c = e / kFH, h = e % kFH;
    const __nv_bfloat16 v = W1[e];
    S.w1[c * kLd2 + h] = v;
    S.w1t[h * kLd1 + c] = v;
  }
  for (int e = tid; e < kFH * kFH; e += blockDim.x) {
    const int i = e / kFH, o = e % kFH;
    const __nv_bfloat16 v = W2[e];
    S.w2[i * kLd2 + o] = v;
    S.w2t[o * kLd2 + i] = v;
  }
  for (int e = tid; e < kFH; e += blockDim.x) {
    S.b1[e] = b1[e];
    S.b2[e] = b2[e];
    S.w3[e] = w3[e];
  }
  __syncthreads();
  const int warp = tid >> 5, lane = tid & 31;
  const int g = lane >> 2, q = lane & 3;
  const float bias3 = b3[0];
  const int n_blocks = (n_atoms + 15) / 16;
  const int wpb = blockDim.x >> 5;
  for (int blk = blockIdx.x * wpb + warp; blk < n_blocks;
       blk += gridDim.x * wpb) {
    const int r0 = blk * 16;
    const int ra = r0 + g, rb = r0 + g + 8;
    const bool va = ra < n_atoms, vb = rb < n_atoms;
    // A fragments of X (2 k-tiles of 16 descriptors)
    unsigned xa[2][4];
#pragma unroll
    for (int t = 0; t < 2; ++t) {
      const int k = 16 * t + 2 * q;
      xa[t][0] = va ? ld_u32(X + (size_t)ra * kFC + k) : 0u;
      xa[t][1] = vb ? ld_u32(X + (size_t)rb * kFC + k) : 0u;
      xa[t][2] = va ? ld_u32(X + (size_t)ra * kFC + k + 8) : 0u;
      xa[t][3] = vb ? ld_u32(X + (size_t)rb * kFC + k + 8) : 0u;
    }
    // layer 1: z1 [16 x 128] -> h1 as A fragments (8 k-tiles)
    unsigned h1[8][4];
#pragma unroll
    for (int j = 0; j < 16; j += 2) {
      float c0[4] = {0.f, 0.f, 0.f, 0.f}, c1[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int t = 0; t < 2; ++t) {
        const __nv_bfloat16 *p0 = S.w1t + (8 * j + g) * kLd1 + 16 * t + 2 * q;
        const __nv_bfloat16 *p1 = p0 + 8 * kLd1;
        const unsigned bb0[2] = {ld_u32(p0), ld_u32(p0 + 8)};
        const unsigned bb1[2] = {ld_u32(p1), ld_u32(p1 + 8)};
        mma_bf16_16816(c0, xa[t], bb0);
        mma_bf16_16816(c1, xa[t], bb1);
      }
      const int n0 = 8 * j + 2 * q, n1 = n0 + 8;
      h1[j / 2][0] = pack2f(silu_f(c0[0] + S.b1[n0]), silu_f(c0[1] + S.b1[n0 + 1]));
      h1[j / 2][1] = pack2f(silu_f(c0[2] + S.b1[n0]), silu_f(c0[3] + S.b1[n0 + 1]));
      h1[j / 2][2] = pack2f(silu_f(c1[0] + S.b1[n1]), silu_f(c1[1] + S.b1[n1 + 1]));
      h1[j / 2][3] = pack2f(silu_f(c1[2] + S.b1[n1]), silu_f(c1[3] + S.b1[n1 + 1]));
    }
    // layer 2 (z2 kept for the backward pass), output y
    float z2[16][4];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
#pragma unroll
      for (int e = 0; e < 4; ++e) z2[j][e] = 0.f;
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const __nv_bfloat16 *p = S.w2t + (8 * j + g) * kLd2 + 16 * t + 2 * q;
        const unsigned bb[2] = {ld_u32(p), ld_u32(p + 8)};
        mma_bf16_16816(z2[j], h1[t], bb);
      }
    }
    float ya = 0.f, yb = 0.f;
    unsigned dz2[8][4];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const int n = 8 * j + 2 * q;
      float d[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int col = n + (e & 1);
        const float z = z2[j][e] + S.b2[col];
        const float w = S.w3[col];
        if (e < 2) ya = fmaf(silu_f(z), w, ya); else yb = fmaf(silu_f(z), w, yb);
        d[e] = w * dsilu_f(z);
      }
      if ((j & 1) == 0) {
        dz2[j / 2][0] = pack2f(d[0], d[1]);
        dz2[j / 2][1] = pack2f(d[2], d[3]);
      } else {
        dz2[j / 2][2] = pack2f(d[0], d[1]);
        dz2[j / 2][3] = pack2f(d[2], d[3]);
      }
    }
    ya += __shfl_xor_sync(0xffffffffu, ya, 1);
    ya += __shfl_xor_sync(0xffffffffu, ya, 2);
    yb += __shfl_xor_sync(0xffffffffu, yb, 1);
    yb += __shfl_xor_sync(0xffffffffu, yb, 2);
    if (q == 0) {
      if (va) y[ra] = ya + bias3;
      if (vb) y[rb] = yb + bias3;
    }
    // dh1 = dz2 W2^T, then dz1 = dh1 * silu'(z1) (z1 recomputed per tile),
    // packed as A fragments of the last product
    unsigned dz1[8][4];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const __nv_bfloat16 *p = S.w2 + (8 * j + g) * kLd2 + 16 * t + 2 * q;
        const unsigned bb[2] = {ld_u32(p), ld_u32(p + 8)};
        mma_bf16_16816(acc, dz2[t], bb);
      }
      float z1[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int t = 0; t < 2; ++t) {
        const __nv_bfloat16 *p = S.w1t + (8 * j + g) * kLd1 + 16 * t + 2 * q;
        const unsigned bb[2] = {ld_u32(p), ld_u32(p + 8)};
        mma_bf16_16816(z1, xa[t], bb);
      }
      const int n = 8 * j + 2 * q;
      float d[4];
#pragma unroll
      for (int e = 0; e < 4; ++e)
        d[e] = acc[e] * dsilu_f(z1[e] + S.b1[n + (e & 1)]);
      if ((j & 1) == 0) {
        dz1[j / 2][0] = pack2f(d[0], d[1]);
        dz1[j / 2][1] = pack2f(d[2], d[3]);
      } else {
        dz1[j / 2][2] = pack2f(d[0], d[1]);
        dz1[j / 2][3] = pack2f(d[2], d[3]);
      }
    }
    // g = dz1 W1^T  [16 x 32]
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const __nv_bfloat16 *p = S.w1 + (8 * j + g) * kLd2 + 16 * t + 2 * q;
        const unsigned bb[2] = {ld_u32(p), ld_u32(p + 8)};
        mma_bf16_16816(acc, dz1[t], bb);
      }
      const int c = 8 * j + 2 * q;
      if (va)
        *reinterpret_cast<__half2 *>(gout + (size_t)ra * kFC + c) =
            __floats2half2_rn(acc[0], acc[1]);
      if (vb)
        *reinterpret_cast<__half2 *>(gout + (size_t)rb * kFC + c) =
            __floats2half2_rn(acc[2], acc[3]);
    }
  }
}

__global__ void to_bf16_kernel(const float *__restrict__ x, size_t n,
                               __nv_bfloat16 *__restrict__ y) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    y[i] = __float2bfloat16_rn(x[i]);
}

}  // namespace pyiid
