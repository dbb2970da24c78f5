// debye_kernels.cuh -- pair-tiled Debye kernels for sm_103a.
//
// Atoms of every configuration are sorted by species and cut into tiles of at
// most kTile atoms that never straddle a (configuration, species) boundary, so
// every tile pair has one species pair and the form factors factor out of the
// pair loops:
//   S_k = sum_{sa>=sb} f_sa(Q_k) f_sb(Q_k) D^{sa sb}_k,
//   D^{sa sb}_k = sum over pairs of that species pair of sin(Q_k r)/r.
// The kernels therefore never read form factors in their inner loops; the
// small finishing kernels apply them.
//
// Reference formulas restated (pyIID, pyiid/experiments/elasticscatter/):
//   pair vectors and distances      kernels/cpu_flat.py:16-52
//                                   (GPU twin kernels/gpu_flat.py:11-49)
//   f_i f_j normalisation array     kernels/cpu_flat.py:57-74
//   omega = sin(Q r)/r, F terms     kernels/cpu_flat.py:79-114, gpu_flat.py:73-112
//   gradient of omega and of F      kernels/cpu_flat.py:122-194, gpu_flat.py:116-166
//   gradient scatter (signs)        kernels/cpu_experimental.py:8-15
//   sums, na, x2, nan_to_num        cpu_wrappers/flat_multi_cpu_wrap.py:22-102
//   Rw / chi^2 gradients (adjoint)  kernels/master_kernel.py:293-376, 392-396
#pragma once

#include <cstdint>

#include "pair_math.cuh"

namespace pyiid {

constexpr int kTile = 32;    // atoms per tile
constexpr int kBlock = 256;  // threads per CTA of the pair kernels
constexpr int kJMaxTiles = 32;  // max J tiles per F(Q) work item

// Split of the tiles J of a configuration over gridDim.z = n CTAs per
// (tile I, chunk block), for configurations too small to fill the GPU
// otherwise: CTA z sweeps the z-th of n contiguous parts of the J tiles and
// writes raw partial rows (no NaN mapping) at out + z * out_stride and its
// F(Q) rows at fpart + z * fpart_stride; combine_grad_parts_kernel and the
// finishing kernel add the parts in a fixed order.  n = 1: no split.
constexpr int kMaxJSplit = 8;  // parts of a split (choose_jsplit's bound)
struct JSplit {
  int n;
  size_t out_stride, fpart_stride;
  // part handled by blockIdx.z: the parts with more tiles J first, so that
  // the last wave of CTAs holds the shorter ones
  unsigned char order[kMaxJSplit];
};


// Tile descriptor: start (in sorted order), atom count, configuration, species.
// (stored as int4)

// Triangular index q in [0, n(n-1)/2) -> (a, b), a > b.
__device__ __forceinline__ void tri_index(int q, int &a, int &b) {
  int ai = (int)((1.0f + sqrtf(1.0f + 8.0f * (float)q)) * 0.5f);
  while (ai * (ai - 1) / 2 > q) --ai;
  while ((ai + 1) * ai / 2 <= q) ++ai;
  a = ai;
  b = q - ai * (ai - 1) / 2;
}

__device__ __forceinline__ float4 load_atom(const float *__restrict__ pos,
                                            const int *__restrict__ perm,
                                            int sorted_index) {
  int o = perm[sorted_index];
  return make_float4(pos[3 * o], pos[3 * o + 1], pos[3 * o + 2], 0.f);
}

// ===================================================================== F(Q)
// One CTA per work item (tile I, tiles [J0, J1) of one species pair); CTA b
// takes item order[b] (largest items first, so that the last wave holds the
// small ones; nullptr: item b), and writes partial row `item`.  Thread
// (chunk c, group g) accumulates bins [kbase, kbase+L) over the pairs q = g,
// g + n_groups, ... of every tile pair, NP pairs at a time (independent
// recurrences interleaved for instruction-level parallelism).  Per pair the
// record holds
//   a = (th_hi, th_lo, lambda, sigma)
//   b = (sin_th / r, -lambda / (2 r), 1 / r, 0)
// so that the recurrence runs on t_k = sin(k theta_e) / r directly.
// Per bin and pair: FFMA + FADD (recurrence) + FADD/FFMA (accumulate).
// Per tile pair the FP32 register sums are folded into a Kahan-compensated
// FP32 accumulator kept in shared memory (two floats per bin and thread); the
// CTA reduces its groups in FP64 and writes one partial row.
// Dynamic shared memory: 2*32*32 float4 records + 2*L*blockDim floats; the
// final FP64 reduction reuses the record space (n_chunks*L doubles <= 32 KB).
template <int L>
struct FqSeed {
  float t, v, lam, sig;
};

template <int L>
__device__ __forceinline__ FqSeed<L> fq_seed(const float4 &ra, const float4 &rb,
                                             float kf, float mask) {
  float s0, c0;
  seed_sincos(kf, ra.x, ra.y, s0, c0);
  FqSeed<L> z;
  z.t = mask * (rb.z * s0);
  z.v = mask * fmaf(rb.x, c0, rb.y * s0);
  z.lam = ra.z;
  z.sig = ra.w;
  return z;
}

template <int L, int NP>
__global__ void __launch_bounds__(kBlock, 2)
    fq_pair_kernel(const float *__restrict__ pos, const int *__restrict__ perm,
                   const int4 *__restrict__ tiles,
                   const int4 *__restrict__ items,
                   const int *__restrict__ order, float dq_hi, float dq_lo,
                   int kb0, int n_chunks, int n_groups, int n_bins,
                   double *__restrict__ partial) {
  extern __shared__ float4 smem[];
  float4 *recA = smem;
  float4 *recB = smem + kTile * kTile;
  // per-thread Kahan sum and compensation, [j][thread] (conflict-free)
  float *kS = reinterpret_cast<float *>(smem + 2 * kTile * kTile);
  float *kC = kS + L * blockDim.x;
  __shared__ float4 sI[kTile], sJ[kTile];

  const int item = order ? order[blockIdx.x] : (int)blockIdx.x;
  const int4 it = items[item];
  const int4 ti = tiles[it.x];
  const int tid = threadIdx.x;
  const int c = tid % n_chunks;
  const int g = tid / n_chunks;
  const bool active = g < n_groups;
  const int kbase = kb0 + (blockIdx.y * n_chunks + c) * L;
  const float kf = (float)kbase;

  if (tid < ti.y) sI[tid] = load_atom(pos, perm, ti.x + tid);

#pragma unroll
  for (int j = 0; j < L; ++j) {
    kS[j * blockDim.x + tid] = 0.f;
    kC[j * blockDim.x + tid] = 0.f;
  }

  for (int tj = it.y; tj < it.z; ++tj) {
    const int4 tJ = tiles[tj];
    __syncthreads();
    if (tid < tJ.y) sJ[tid] = load_atom(pos, perm, tJ.x + tid);
    __syncthreads();
    const bool diag = (tj == it.x);
    const int np = diag ? ti.y * (ti.y - 1) / 2 : ti.y * tJ.y;
    for (int q = tid; q < np; q += blockDim.x) {
      int a, b;
      if (diag) {
        tri_index(q, a, b);
      } else {
        a = q / tJ.y;
        b = q - a * tJ.y;
      }
      const float4 pa = sI[a];
      const float4 pb = diag ? sI[b] : sJ[b];
      float dx, dy, dz;
      PairPhase p = pair_phase(pa.x, pa.y, pa.z, pb.x, pb.y, pb.z, dq_hi,
                               dq_lo, dx, dy, dz);
      recA[q] = make_float4(p.th_hi, p.th_lo, p.lam, p.sigma);
      recB[q] = make_float4(p.sin_th * p.inv_r, -0.5f * p.lam * p.inv_r,
                            p.inv_r, 0.f);
    }
    __syncthreads();
    if (active && np > 0) {
      float acc[L];
#pragma unroll
      for (int j = 0; j < L; ++j) acc[j] = 0.f;
      for (int q = g; q < np; q += NP * n_groups) {
        FqSeed<L> z[NP];
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          const int qq = q + p * n_groups;
          const int qc = qq < np ? qq : np - 1;
          z[p] = fq_seed<L>(recA[qc], recB[qc], kf, qq < np ? 1.f : 0.f);
        }
#pragma unroll
        for (int p = 0; p < NP; ++p) acc[0] += z[p].t;
#pragma unroll
        for (int j = 1; j < L; ++j) {
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            z[p].v = fmaf(z[p].lam, z[p].t, z[p].v);
            z[p].t = z[p].t + z[p].v;
            if (j & 1)
              acc[j] = fmaf(z[p].t, z[p].sig, acc[j]);
            else
              acc[j] += z[p].t;
          }
        }
      }
#pragma unroll
      for (int j = 0; j < L; ++j) {
        const float Sj = kS[j * blockDim.x + tid];
        const float y = __fsub_rn(acc[j], kC[j * blockDim.x + tid]);
        const float s = __fadd_rn(Sj, y);
        kC[j * blockDim.x + tid] = __fsub_rn(__fsub_rn(s, Sj), y);
        kS[j * blockDim.x + tid] = s;
      }
    }
  }

  // reduce the groups of each chunk in FP64 (the record buffer is dead now)
  __syncthreads();
  double *red = reinterpret_cast<double *>(smem);
  for (int gg = 0; gg < n_groups; ++gg) {
    if (active && g == gg) {
#pragma unroll
      for (int j = 0; j < L; ++j) {
        const double v = (double)kS[j * blockDim.x + tid] -
                         (double)kC[j * blockDim.x + tid];
        red[c * L + j] = (gg == 0) ? v : red[c * L + j] + v;
      }
    }
    __syncthreads();
  }
  const int nk = n_chunks * L;
  const int kfirst = kb0 + blockIdx.y * nk;
  double *out = partial + (size_t)item * n_bins;
  for (int i = tid; i < nk; i += blockDim.x) {
    const int k = kfirst + i;
    if (k < n_bins) out[k] = red[i];
  }
}

// F_k = 2 * nan_to_num(float(S_k) / float(na_k)): the reference divides
// float32 by float32 and nan_to_num's the result (+-inf -> +-FLT_MAX).
__device__ __forceinline__ float fq_value(double s, double na) {
  float v = (float)s / (float)na;
  if (isnan(v)) v = 0.f;
  if (isinf(v)) v = v > 0.f ? 3.402823466e38f : -3.402823466e38f;
  float outv = 2.0f * v;
  if (isinf(outv)) outv = outv > 0.f ? 3.402823466e38f : -3.402823466e38f;
  return outv;
}

// Finishing kernel for F(Q): for configuration b and bin k
//   S_k  = sum_sp f_sa f_sb sum_{items of key (b, sp)} partial[item][k]
//   F_k  = 2 * nan_to_num(float(S_k / na_k))
// as wrap_fq does (cpu_wrappers/flat_multi_cpu_wrap.py:44-60: FP64 sum of the
// FP32 pair terms, na = N mean_{i>j} f_i f_j, factor 2, nan_to_num).
// na is precomputed per (config, bin) on the host in FP64 (it depends only on
// species counts and form factors).  Configurations with < 2 atoms give 0.
__global__ void fq_finish_kernel(const double *__restrict__ partial,
                                 const int *__restrict__ key_item_begin,
                                 const float *__restrict__ ftab,
                                 const int2 *__restrict__ spair_species,
                                 const double *__restrict__ na, int n_spairs,
                                 int n_bins, int kb_out, float *__restrict__ fq,
                                 double *__restrict__ fq_raw) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (k >= n_bins) return;
  float outv = 0.f;
  double sraw = 0.0;
  if (k >= kb_out) {
    double s = 0.0;
    for (int sp = 0; sp < n_spairs; ++sp) {
      const int key = b * n_spairs + sp;
      const int i0 = key_item_begin[key], i1 = key_item_begin[key + 1];
      if (i0 == i1) continue;
      double d = 0.0;
      for (int i = i0; i < i1; ++i) d += partial[(size_t)i * n_bins + k];
      const int2 ss = spair_species[sp];
      s += (double)ftab[ss.x * n_bins + k] * (double)ftab[ss.y * n_bins + k] *
           d;
    }
    sraw = s;
    outv = fq_value(s, na[(size_t)b * n_bins + k]);
  }
  if (fq) fq[(size_t)b * n_bins + k] = outv;
  if (fq_raw) fq_raw[(size_t)b * n_bins + k] = sraw;
}

// ==================================================================== dF/dx
// The value of wrap_fq_grad (cpu_wrappers/flat_multi_cpu_wrap.py:63-102):
// row a = -(1/na) sum_b f_a f_b (Q cos(Q r) - sin(Q r)/r)/r^2 (x_a - x_b),
// i.e. -1/2 dF/dx_a (kernels/cpu_flat.py:122-194 with the scatter signs of
// kernels/cpu_experimental.py:8-15; no factor 2, nan_to_num of the rows).
// Owner-computes: CTA (tile I, chunk block) with threads (atom a, chunk cl);
// every thread sweeps all tiles J of its configuration and accumulates the
// 3 x L gradient bins of its atom, so no atomics or partials are needed.
// Records per (a in I, b in J), stored [b][a] so the few atoms of a warp read
// adjacent records (no bank conflicts):
//   a = (th_hi, th_lo, lambda, sigma)
//   b = (beta sin_th, -beta lambda / 2, beta, gamma')   beta = -1/r^3,
//                                                        gamma' = -r dq/(2 sin_th)
//   c = (dx, dy, dz, 0)
// With t, v scaled by beta, per bin
//   g_k = sigma^k (k gamma' (v_k + v_{k+1}) + t_k) = (Q_k cos(Q_k r) - sin(Q_k r)/r)/r^2.
// Per bin and ordered pair: 2 (recurrence) + 1 (u) + 1 (k gamma') + 1 (g) +
// 3 (accumulate) = 8 FP32 instructions.  NP pairs are interleaved per thread.
// At every species change of J (and at the end) the thread folds
// coef[b][sa][sb][k] * acc into its own output rows.
struct GradState {
  float t, v, kg, gam, lam, dx, dy, dz, sx, sy, sz;
};

__device__ __forceinline__ GradState grad_seed(const float4 &ra,
                                               const float4 &rb,
                                               const float4 &rc, float kf) {
  float s0, c0;
  seed_sincos(kf, ra.x, ra.y, s0, c0);
  GradState z;
  z.t = rb.z * s0;
  z.v = fmaf(rb.x, c0, rb.y * s0);
  z.kg = kf * rb.w;
  z.gam = rb.w;
  z.lam = ra.z;
  z.dx = rc.x;
  z.dy = rc.y;
  z.dz = rc.z;
  z.sx = ra.w * rc.x;
  z.sy = ra.w * rc.y;
  z.sz = ra.w * rc.z;
  return z;
}

template <int L, int CPC, int NP, int MINB>
__global__ void __launch_bounds__(kTile * CPC, MINB)
    gradfq_kernel(const float *__restrict__ pos, const int *__restrict__ perm,
                  const int4 *__restrict__ tiles,
                  const int2 *__restrict__ cfg_tiles, float dq_hi,
                  float dq_lo, int kb0, int chunks_total, int n_bins,
                  const float *__restrict__ coef, int n_species,
                  float *__restrict__ out, JSplit /*no split: n == 1*/) {
  extern __shared__ float4 smem[];
  float4 *recA = smem;
  float4 *recB = smem + kTile * kTile;
  float4 *recC = smem + 2 * kTile * kTile;
  __shared__ float4 sI[kTile], sJ[kTile];

  const int4 ti = tiles[blockIdx.x];
  const int2 ct = cfg_tiles[ti.z];
  const int tid = threadIdx.x;
  const int al = tid / CPC;
  const int chunk = blockIdx.y * CPC + tid % CPC;
  const bool active = (al < ti.y) && (chunk < chunks_total);
  const int kbase = kb0 + chunk * L;
  const float kf = (float)kbase;

  if (tid < ti.y) sI[tid] = load_atom(pos, perm, ti.x + tid);

  float ax[L], ay[L], az[L];
#pragma unroll
  for (int j = 0; j < L; ++j) {
    ax[j] = 0.f;
    ay[j] = 0.f;
    az[j] = 0.f;
  }
  int cur_sb = -1;
  bool first_flush = true;
  const int out_row = active ? perm[ti.x + al] : 0;

  auto flush = [&](int sb, bool last) {
    if (!active) return;
    const float *cf =
        coef + (((size_t)ti.z * n_species + ti.w) * n_species + sb) * n_bins;
    float *o = out + (size_t)out_row * 3 * n_bins;
#pragma unroll
    for (int j = 0; j < L; ++j) {
      const int k = kbase + j;
      if (k < n_bins) {
        const float w = cf[k];
        float vx = w * ax[j], vy = w * ay[j], vz = w * az[j];
        if (!first_flush) {
          vx += o[k];
          vy += o[n_bins + k];
          vz += o[2 * n_bins + k];
        }
        if (last) {
          vx = isnan(vx) ? 0.f : (isinf(vx) ? copysignf(3.402823466e38f, vx) : vx);
          vy = isnan(vy) ? 0.f : (isinf(vy) ? copysignf(3.402823466e38f, vy) : vy);
          vz = isnan(vz) ? 0.f : (isinf(vz) ? copysignf(3.402823466e38f, vz) : vz);
        }
        o[k] = vx;
        o[n_bins + k] = vy;
        o[2 * n_bins + k] = vz;
      }
      ax[j] = 0.f;
      ay[j] = 0.f;
      az[j] = 0.f;
    }
    first_flush = false;
  };

  for (int tj = ct.x; tj < ct.y; ++tj) {
    const int4 tJ = tiles[tj];
    if (cur_sb >= 0 && tJ.w != cur_sb) flush(cur_sb, false);
    cur_sb = tJ.w;
    __syncthreads();
    if (tid < tJ.y) sJ[tid] = load_atom(pos, perm, tJ.x + tid);
    __syncthreads();
    const bool same = (tj == (int)blockIdx.x);
    for (int q = tid; q < kTile * kTile; q += blockDim.x) {
      const int b = q / kTile, a = q % kTile;
      float4 ra = make_float4(0.f, 0.f, 0.f, 1.f);
      float4 rb = make_float4(0.f, 0.f, 0.f, 0.f);
      float4 rc = make_float4(0.f, 0.f, 0.f, 0.f);
      if (a < ti.y && b < tJ.y && !(same && a == b)) {
        const float4 pa = sI[a];
        const float4 pb = sJ[b];
        float dx, dy, dz;
        PairPhase p = pair_phase(pa.x, pa.y, pa.z, pb.x, pb.y, pb.z, dq_hi,
                                 dq_lo, dx, dy, dz);
        const float beta = -(p.inv_r * p.inv_r * p.inv_r);
        const float gam = -p.r * dq_hi / (2.0f * p.sin_th);
        ra = make_float4(p.th_hi, p.th_lo, p.lam, p.sigma);
        rb = make_float4(beta * p.sin_th, -0.5f * p.lam * beta, beta, gam);
        rc = make_float4(dx, dy, dz, 0.f);
      }
      recA[q] = ra;
      recB[q] = rb;
      recC[q] = rc;
    }
    __syncthreads();
    if (active) {
      // records beyond tJ.y are zero, so the NP-wide loop may run past it
      for (int b = 0; b < tJ.y; b += NP) {
        GradState z[NP];
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          const int q = (b + p) * kTile + al;
          z[p] = grad_seed(recA[q], recB[q], recC[q], kf);
        }
#pragma unroll
        for (int j = 0; j < L; ++j) {
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            const float vn = fmaf(z[p].lam, z[p].t, z[p].v);
            const float u = z[p].v + vn;
            const float gk = fmaf(z[p].kg, u, z[p].t);
            if (j & 1) {
              ax[j] = fmaf(gk, z[p].sx, ax[j]);
              ay[j] = fmaf(gk, z[p].sy, ay[j]);
              az[j] = fmaf(gk, z[p].sz, az[j]);
            } else {
              ax[j] = fmaf(gk, z[p].dx, ax[j]);
              ay[j] = fmaf(gk, z[p].dy, ay[j]);
              az[j] = fmaf(gk, z[p].dz, az[j]);
            }
            z[p].t = z[p].t + vn;
            z[p].v = vn;
            z[p].kg += z[p].gam;
          }
        }
      }
    }
  }
  if (cur_sb >= 0) flush(cur_sb, true);
}

// ============================================ packed (FP32x2) pair kernels
// Same work decomposition as the kernels above, on the even/odd formulation
// of pair_math.cuh: one packed instruction advances bins k and k+1.
// F(Q) per two bins and pair: FFMA2 + FFMA2 (recurrence) + FADD2/FFMA2.
// Records: a = (th_hi, th_lo, kappa, sigma2), b = (ch/r, sin theta, 1/r,
// cos theta); sh/r is (kappa/2)/r, and the odd slot's seed is the even one
// rotated by theta (seed_sincos2r).
// NP = 2: each thread advances two pairs together (independent recurrence
// chains for the FMA pipe; the two-FMA dependency of one chain is what
// limits NP = 1); a missing second pair has zero records.
template <int L, int NP = 1>
__global__ void __launch_bounds__(kBlock, 2)
    fq_pair2_kernel(const float *__restrict__ pos, const int *__restrict__ perm,
                    const int4 *__restrict__ tiles,
                    const int4 *__restrict__ items,
                   const int *__restrict__ order, float dq_hi, float dq_lo,
                    int kb0, int n_chunks, int n_groups, int n_bins,
                    double *__restrict__ partial) {
  static_assert(L % 2 == 0, "L must be even");
  constexpr int M = L / 2;
  extern __shared__ float4 smem[];
  float4 *recA = smem;
  float4 *recB = smem + kTile * kTile;
  float *kS = reinterpret_cast<float *>(smem + 2 * kTile * kTile);
  float *kC = kS + L * blockDim.x;
  __shared__ float4 sI[kTile], sJ[kTile];

  const int item = order ? order[blockIdx.x] : (int)blockIdx.x;
  const int4 it = items[item];
  const int4 ti = tiles[it.x];
  const int tid = threadIdx.x;
  const int c = tid % n_chunks;
  const int g = tid / n_chunks;
  const bool active = g < n_groups;
  const int kbase = kb0 + (blockIdx.y * n_chunks + c) * L;
  const float kf = (float)kbase;

  if (tid < ti.y) sI[tid] = load_atom(pos, perm, ti.x + tid);
#pragma unroll
  for (int j = 0; j < L; ++j) {
    kS[j * blockDim.x + tid] = 0.f;
    kC[j * blockDim.x + tid] = 0.f;
  }

  for (int tj = it.y; tj < it.z; ++tj) {
    const int4 tJ = tiles[tj];
    __syncthreads();
    if (tid < tJ.y) sJ[tid] = load_atom(pos, perm, tJ.x + tid);
    __syncthreads();
    const bool diag = (tj == it.x);
    const int np = diag ? ti.y * (ti.y - 1) / 2 : ti.y * tJ.y;
    for (int q = tid; q < np; q += blockDim.x) {
      int a, b;
      if (diag) {
        tri_index(q, a, b);
      } else {
        a = q / tJ.y;
        b = q - a * tJ.y;
      }
      const float4 pa = sI[a];
      const float4 pb = diag ? sI[b] : sJ[b];
      float dx, dy, dz;
      PairPhase2 p = pair_phase2(pa.x, pa.y, pa.z, pb.x, pb.y, pb.z, dq_hi,
                                 dq_lo, dx, dy, dz);
      recA[q] = make_float4(p.th_hi, p.th_lo, p.kappa, p.sigma2);
      recB[q] = make_float4(p.ch * p.inv_r, p.sth, p.inv_r, p.cth);
    }
    __syncthreads();
    if (active && np > 0) {
      float2 acc[M];
#pragma unroll
      for (int m = 0; m < M; ++m) acc[m] = f2(0.f);
      for (int q = g; q < np; q += NP * n_groups) {
        float2 t[NP], w[NP], kp[NP], km[NP], sg[NP];
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          const int qq = q + p * n_groups;
          const bool ok = qq < np;
          const float4 ra = recA[ok ? qq : q];
          const float4 rb = ok ? recB[qq] : make_float4(0.f, 0.f, 0.f, 0.f);
          float2 s, co;
          seed_sincos2r(kf, ra.x, ra.y, rb.y, rb.w, s, co);
          // sh / r = (kappa / 2) / r, bitwise the product the record held
          const float shr = __fmul_rn(0.5f * ra.z, rb.z);
          t[p] = __fmul2_rn(f2(rb.z), s);
          w[p] = __ffma2_rn(co, f2(rb.x), __fmul2_rn(s, f2(shr)));
          kp[p] = f2(ra.z);
          km[p] = f2(-ra.z);
          sg[p] = f2(ra.w);
        }
#pragma unroll
        for (int m = 0; m < M; ++m) {
#pragma unroll
          for (int p = 0; p < NP; ++p)
            acc[m] = (m & 1) ? __ffma2_rn(t[p], sg[p], acc[m])
                             : __fadd2_rn(acc[m], t[p]);
          if (m + 1 < M) {
#pragma unroll
            for (int p = 0; p < NP; ++p) {
              w[p] = __ffma2_rn(km[p], t[p], w[p]);
              t[p] = __ffma2_rn(kp[p], w[p], t[p]);
            }
          }
        }
      }
#pragma unroll
      for (int m = 0; m < M; ++m) {
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const int j = 2 * m + e;
          const float a = e ? acc[m].y : acc[m].x;
          const float Sj = kS[j * blockDim.x + tid];
          const float y = __fsub_rn(a, kC[j * blockDim.x + tid]);
          const float sum = __fadd_rn(Sj, y);
          kC[j * blockDim.x + tid] = __fsub_rn(__fsub_rn(sum, Sj), y);
          kS[j * blockDim.x + tid] = sum;
        }
      }
    }
  }
  __syncthreads();
  double *red = reinterpret_cast<double *>(smem);
  for (int gg = 0; gg < n_groups; ++gg) {
    if (active && g == gg) {
#pragma unroll
      for (int j = 0; j < L; ++j) {
        const double v = (double)kS[j * blockDim.x + tid] -
                         (double)kC[j * blockDim.x + tid];
        red[c * L + j] = (gg == 0) ? v : red[c * L + j] + v;
      }
    }
    __syncthreads();
  }
  const int nk = n_chunks * L;
  const int kfirst = kb0 + blockIdx.y * nk;
  double *out = partial + (size_t)item * n_bins;
  for (int i = tid; i < nk; i += blockDim.x) {
    const int k = kfirst + i;
    if (k < n_bins) out[k] = red[i];
  }
}

// Floats of the record / group-scratch region of fq_pair3_kernel: the two
// record arrays, or the group sums n_groups * n_chunks * (L + 1) <=
// kBlock * (L + 1) (rows padded to the odd stride L + 1: the chunks of a
// warp then fall on distinct banks).
__host__ __device__ constexpr int fq3_scratch_floats(int L) {
  return kBlock * (L + 1) > 2 * kTile * kTile * 4 ? kBlock * (L + 1)
                                                  : 2 * kTile * kTile * 4;
}

// F(Q) pair sums with the group reduction done per tile pair: after each
// tile pair the groups' FP32 register sums go through the (then idle)
// record buffer, are added in a fixed order and accumulated per bin in FP64
// shared memory.  No per-thread compensated sums are kept, so the kernel
// fits MINB CTAs per SM (e.g. 4 x 256 threads at <= 64 registers) instead
// of two.  Dynamic shared memory: fq3_scratch_floats(L) floats of records
// and group scratch + n_chunks * L doubles.
// One work unit: work item `item` (tile I against a run of tiles J), bin
// block yb (n_chunks * L bins), written to partial row `item`.
template <int L>
__device__ __forceinline__ void fq_pair3_unit(
    const float *__restrict__ pos, const int *__restrict__ perm,
    const int4 *__restrict__ tiles, const int4 *__restrict__ items, int item,
    int yb, float dq_hi, float dq_lo, int kb0, int n_chunks, int n_groups,
    int n_bins, double *__restrict__ partial) {
  static_assert(L % 2 == 0, "L must be even");
  constexpr int M = L / 2;
  extern __shared__ float4 smem[];
  float4 *recA = smem;
  float4 *recB = smem + kTile * kTile;
  float *scratch = reinterpret_cast<float *>(smem);
  double *acc64 = reinterpret_cast<double *>(scratch + fq3_scratch_floats(L));
  __shared__ float4 sI[kTile], sJ[kTile];

  const int4 it = items[item];
  const int4 ti = tiles[it.x];
  const int tid = threadIdx.x;
  const int c = tid % n_chunks;
  const int g = tid / n_chunks;
  const bool active = g < n_groups;
  const int kbase = kb0 + (yb * n_chunks + c) * L;
  const float kf = (float)kbase;
  const int nk = n_chunks * L;

  if (tid < ti.y) sI[tid] = load_atom(pos, perm, ti.x + tid);
  for (int i = tid; i < nk; i += blockDim.x) acc64[i] = 0.0;

  for (int tj = it.y; tj < it.z; ++tj) {
    const int4 tJ = tiles[tj];
    __syncthreads();
    if (tid < tJ.y) sJ[tid] = load_atom(pos, perm, tJ.x + tid);
    __syncthreads();
    const bool diag = (tj == it.x);
    const int np = diag ? ti.y * (ti.y - 1) / 2 : ti.y * tJ.y;
    for (int q = tid; q < np; q += blockDim.x) {
      int a, b;
      if (diag) {
        tri_index(q, a, b);
      } else {
        a = q / tJ.y;
        b = q - a * tJ.y;
      }
      const float4 pa = sI[a];
      const float4 pb = diag ? sI[b] : sJ[b];
      float dx, dy, dz;
      PairPhase2 p = pair_phase2(pa.x, pa.y, pa.z, pb.x, pb.y, pb.z, dq_hi,
                                 dq_lo, dx, dy, dz);
      recA[q] = make_float4(p.th_hi, p.th_lo, p.kappa, p.sigma2);
      recB[q] = make_float4(p.ch * p.inv_r, p.sth, p.inv_r, p.cth);
    }
    __syncthreads();
    float2 acc[M];
#pragma unroll
    for (int m = 0; m < M; ++m) acc[m] = f2(0.f);
    if (active) {
      for (int q = g; q < np; q += n_groups) {
        const float4 ra = recA[q];
        const float4 rb = recB[q];
        float2 s, co;
        seed_sincos2r(kf, ra.x, ra.y, rb.y, rb.w, s, co);
        const float shr = __fmul_rn(0.5f * ra.z, rb.z);
        float2 t = __fmul2_rn(f2(rb.z), s);
        float2 w = __ffma2_rn(co, f2(rb.x), __fmul2_rn(s, f2(shr)));
        const float2 kp = f2(ra.z), km = f2(-ra.z), sg = f2(ra.w);
#pragma unroll
        for (int m = 0; m < M; ++m) {
          acc[m] = (m & 1) ? __ffma2_rn(t, sg, acc[m]) : __fadd2_rn(acc[m], t);
          if (m + 1 < M) {
            w = __ffma2_rn(km, t, w);
            t = __ffma2_rn(kp, w, t);
          }
        }
      }
    }
    __syncthreads();  // records are dead: reuse them as group scratch
    constexpr int Lp = L + 1;
    const int nkp = n_chunks * Lp;
    if (active) {
#pragma unroll
      for (int m = 0; m < M; ++m) {
        scratch[g * nkp + c * Lp + 2 * m] = acc[m].x;
        scratch[g * nkp + c * Lp + 2 * m + 1] = acc[m].y;
      }
    }
    __syncthreads();
    for (int i = tid; i < nk; i += blockDim.x) {
      const int off = (i / L) * Lp + i % L;
      float sum = 0.f;
      for (int gg = 0; gg < n_groups; ++gg) sum += scratch[gg * nkp + off];
      acc64[i] += (double)sum;
    }
  }
  __syncthreads();
  const int kfirst = kb0 + yb * nk;
  double *out = partial + (size_t)item * n_bins;
  for (int i = tid; i < nk; i += blockDim.x) {
    const int k = kfirst + i;
    if (k < n_bins) out[k] = acc64[i];
  }
}

// One CTA per work unit: blockIdx.x = position in `order` (largest items
// first), blockIdx.y = bin block.
template <int L, int MINB>
__global__ void __launch_bounds__(kBlock, MINB)
    fq_pair3_kernel(const float *__restrict__ pos, const int *__restrict__ perm,
                    const int4 *__restrict__ tiles,
                    const int4 *__restrict__ items,
                    const int *__restrict__ order, float dq_hi, float dq_lo,
                    int kb0, int n_chunks, int n_groups, int n_bins,
                    double *__restrict__ partial) {
  const int item = order ? order[blockIdx.x] : (int)blockIdx.x;
  fq_pair3_unit<L>(pos, perm, tiles, items, item, blockIdx.y, dq_hi, dq_lo,
                   kb0, n_chunks, n_groups, n_bins, partial);
}

// Persistent form: as many CTAs as fit on the device at once, each taking
// work units u = 0, 1, ... (item order[u / n_cb], bin block u % n_cb) from
// a device counter (*counter = 0 at launch) until none is left.  The
// partial rows, and so the fixed-order reduction behind them, are those of
// fq_pair3_kernel: results are bitwise equal.
template <int L, int MINB>
__global__ void __launch_bounds__(kBlock, MINB)
    fq_pair3_persistent(const float *__restrict__ pos,
                        const int *__restrict__ perm,
                        const int4 *__restrict__ tiles,
                        const int4 *__restrict__ items,
                        const int *__restrict__ order, float dq_hi,
                        float dq_lo, int kb0, int n_chunks, int n_groups,
                        int n_bins, int n_cb, int n_units, int *counter,
                        double *__restrict__ partial) {
  __shared__ int s_unit;
  while (true) {
    // (the previous unit's last shared-memory reads are behind this
    // barrier pair as well)
    if (threadIdx.x == 0) s_unit = atomicAdd(counter, 1);
    __syncthreads();
    const int u = s_unit;
    __syncthreads();
    if (u >= n_units) break;
    const int j = u / n_cb;
    fq_pair3_unit<L>(pos, perm, tiles, items, order ? order[j] : j, u % n_cb,
                     dq_hi, dq_lo, kb0, n_chunks, n_groups, n_bins, partial);
  }
}

// dF/dx, packed.  Records per (a, b), stored [b][a]:
//   a = (th_hi, th_lo, kappa, sigma2)
//   b = (beta ch, sin theta, beta, gamma')   beta = -1/r^3,
//                                            gamma' = -r dq/(2 ch)
//   c = (dx, dy, dz, -r^2 with F(Q), else cos theta)
// beta sh = (kappa/2) beta is rebuilt from a and b; with F(Q), cos theta
// sits in a fourth array d.  The odd slot's seed is the even one rotated by
// theta (seed_sincos2r).
// Per two bins and ordered pair: FFMA2 (w) + FADD2 (u) + FFMA2 (g) +
// 3 FFMA2 (accumulate) + FFMA2 (t) + FADD2 (k gamma') = 8 instructions.
//
// WITH_F also returns the F(Q) pair sums of the same pass.  The recurrence
// variable t_m = beta sin(phi + m theta2) gives the Debye term
// sin(Q_k r)/r = sigma2^m t_m (-r^2): one more FFMA2 per two bins into
// per-thread FP32 sums af, taken only on tiles J >= I so that every
// unordered pair is counted once (the diagonal tile holds both orders of its
// pairs and is weighted 1/2).  Every kFGroup J tiles (at each change of the
// J species, and alone for the diagonal tile) the sums of the warp's atoms
// are combined by shuffles and added, times f_sa f_sb, to the warp's row of
// shared memory with Kahan-compensated FP32 additions (FP64 arithmetic is
// too slow on this part to run per flush); the CTA writes the FP64
// fixed-order sum of its warps' rows to fpart[tile I][k], and
// S_k = sum_I fpart[I][k].
constexpr int kFGroup = 4;
template <bool B>
struct BoolTag {
  static constexpr bool value = B;
};

template <int L, int CPC, bool WITH_F>
__device__ __forceinline__ void gradfq2_body(
    const float *__restrict__ pos, const int *__restrict__ perm,
    const int4 *__restrict__ tiles, const int2 *__restrict__ cfg_tiles,
    float dq_hi, float dq_lo, int kb0, int chunks_total, int n_bins,
    const float *__restrict__ coef, int n_species, float *__restrict__ out,
    const float *__restrict__ ftab, double *__restrict__ fpart, int tile0,
    JSplit js) {
  // tile I of this CTA (tile0: first tile of a part of the tile list)
  const int I = tile0 + (int)blockIdx.x;
  const int part = js.n > 1 ? (int)js.order[blockIdx.z] : 0;
  out += part * js.out_stride;
  if constexpr (WITH_F) fpart += part * js.fpart_stride;
  static_assert(L % 2 == 0, "L must be even");
  static_assert(32 % CPC == 0, "a warp must hold whole atoms");
  constexpr int M = L / 2;
  extern __shared__ float4 smem[];
  float4 *recA = smem;
  float4 *recB = smem + kTile * kTile;
  float4 *recC = smem + 2 * kTile * kTile;
  // pair-only products the chunk threads of a pair would otherwise each
  // form: (sigma2 dx, sigma2 dy, sigma2 dz, sigma2 (-r^2) with F(Q))
  float4 *recE = smem + 3 * kTile * kTile;
  // WITH_F: per warp [CPC][L] FP32 F(Q) sums and their Kahan compensations
  // behind the records
  float *fsum = reinterpret_cast<float *>(smem + 4 * kTile * kTile);
  float *fcmp = fsum + CPC * CPC * L;
  float *recD = fcmp + CPC * CPC * L;  // WITH_F: cos theta of each record
  // positions of tile I and of two tiles J: the next J tile's positions are
  // loaded while the current tile's records are built
  __shared__ float4 sI[kTile], sJb[2][kTile];

  const int4 ti = tiles[I];
  const int2 ct = cfg_tiles[ti.z];
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int al = tid / CPC;
  const int chunk = blockIdx.y * CPC + tid % CPC;
  const bool active = (al < ti.y) && (chunk < chunks_total);
  const int kbase = kb0 + chunk * L;
  const float kf = (float)kbase;

  if (tid < ti.y) sI[tid] = load_atom(pos, perm, ti.x + tid);
  if constexpr (WITH_F)
    for (int i = tid; i < 2 * CPC * CPC * L; i += blockDim.x) fsum[i] = 0.f;

  float2 ax[M], ay[M], az[M];
  float2 af[M];
#pragma unroll
  for (int m = 0; m < M; ++m) {
    ax[m] = f2(0.f);
    ay[m] = f2(0.f);
    az[m] = f2(0.f);
    if constexpr (WITH_F) af[m] = f2(0.f);
  }
  int cur_sb = -1;
  int f_tiles = 0, f_sb = 0;
  bool first_flush = true;
  const int out_row = active ? perm[ti.x + al] : 0;

  auto flush = [&](int sb, bool last) {
    if (!active) return;
    const float *cf =
        coef + (((size_t)ti.z * n_species + ti.w) * n_species + sb) * n_bins;
    float *o = out + (size_t)out_row * 3 * n_bins;
#pragma unroll
    for (int m = 0; m < M; ++m) {
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int k = kbase + 2 * m + e;
        if (k < n_bins) {
          const float w = cf[k];
          float vx = w * (e ? ax[m].y : ax[m].x);
          float vy = w * (e ? ay[m].y : ay[m].x);
          float vz = w * (e ? az[m].y : az[m].x);
          if (!first_flush) {
            vx += o[k];
            vy += o[n_bins + k];
            vz += o[2 * n_bins + k];
          }
          if (last && js.n == 1) {
            vx = isnan(vx) ? 0.f : (isinf(vx) ? copysignf(3.402823466e38f, vx) : vx);
            vy = isnan(vy) ? 0.f : (isinf(vy) ? copysignf(3.402823466e38f, vy) : vy);
            vz = isnan(vz) ? 0.f : (isinf(vz) ? copysignf(3.402823466e38f, vz) : vz);
          }
          o[k] = vx;
          o[n_bins + k] = vy;
          o[2 * n_bins + k] = vz;
        }
      }
      ax[m] = f2(0.f);
      ay[m] = f2(0.f);
      az[m] = f2(0.f);
    }
    first_flush = false;
  };

  // all threads take part (shuffles); lanes < CPC end with their chunk's sum
  auto flush_f = [&](int sb, float scale) {
#pragma unroll
    for (int m = 0; m < M; ++m) {
#pragma unroll
      for (int off = CPC; off < 32; off *= 2) {
        af[m].x += __shfl_xor_sync(0xffffffffu, af[m].x, off);
        af[m].y += __shfl_xor_sync(0xffffffffu, af[m].y, off);
      }
    }
    if (lane < CPC) {
      const int kb = kb0 + (blockIdx.y * CPC + lane) * L;
      const int r0 = (tid >> 5) * CPC * L + lane * L;
      const float *fa = ftab + (size_t)ti.w * n_bins;
      const float *fb = ftab + (size_t)sb * n_bins;
#pragma unroll
      for (int m = 0; m < M; ++m) {
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const int k = kb + 2 * m + e;
          if (k < n_bins) {
            const float y = __fsub_rn(
                __fmul_rn(__fmul_rn(fa[k], fb[k]),
                          scale * (e ? af[m].y : af[m].x)),
                fcmp[r0 + 2 * m + e]);
            const float s0 = fsum[r0 + 2 * m + e];
            const float s1 = __fadd_rn(s0, y);
            fcmp[r0 + 2 * m + e] = __fsub_rn(__fsub_rn(s1, s0), y);
            fsum[r0 + 2 * m + e] = s1;
          }
        }
      }
    }
#pragma unroll
    for (int m = 0; m < M; ++m) af[m] = f2(0.f);
  };

  const int n_cfg_tiles = ct.y - ct.x;
  const int j_end = ct.x + (int)((long long)(part + 1) * n_cfg_tiles / js.n);
  const int j_begin = ct.x + (int)((long long)part * n_cfg_tiles / js.n);
  if (j_begin < j_end) {
    const int4 t0 = tiles[j_begin];
    if (tid < t0.y) sJb[0][tid] = load_atom(pos, perm, t0.x + tid);
  }
  int jb = 0;
  for (int tj = j_begin; tj < j_end; ++tj, jb ^= 1) {
    const int4 tJ = tiles[tj];
    if (cur_sb >= 0 && tJ.w != cur_sb) flush(cur_sb, false);
    if constexpr (WITH_F) {
      if (f_tiles > 0 && (tJ.w != f_sb || f_tiles == kFGroup)) {
        flush_f(f_sb, 1.f);
        f_tiles = 0;
      }
    }
    cur_sb = tJ.w;
    // tile J's positions are in sJb[jb]; the previous tile's loop, its
    // records and sJb[jb ^ 1] are free
    __syncthreads();
    const float4 *sJ = sJb[jb];
    const bool has_next = tj + 1 < j_end;
    int4 tN = make_int4(0, 0, 0, 0);
    float4 pN = make_float4(0.f, 0.f, 0.f, 0.f);
    if (has_next) {
      tN = tiles[tj + 1];
      if (tid < tN.y) pN = load_atom(pos, perm, tN.x + tid);
    }
    const bool same = (tj == I);
    for (int q = tid; q < kTile * kTile; q += blockDim.x) {
      const int b = q / kTile, a = q % kTile;
      float4 ra = make_float4(0.f, 0.f, 0.f, 0.f);
      float4 rb = make_float4(0.f, 0.f, 0.f, 0.f);
      float4 rc = make_float4(0.f, 0.f, 0.f, 0.f);
      float4 re = make_float4(0.f, 0.f, 0.f, 0.f);
      if (a < ti.y && b < tJ.y && !(same && a == b)) {
        const float4 pa = sI[a];
        const float4 pb = sJ[b];
        float dx, dy, dz;
        PairPhase2 p = pair_phase2(pa.x, pa.y, pa.z, pb.x, pb.y, pb.z, dq_hi,
                                   dq_lo, dx, dy, dz);
        const float beta = -(p.inv_r * p.inv_r * p.inv_r);
        const float gam = __fdividef(-p.r * dq_hi, 2.0f * p.ch);  // 2ch in [1.41, 2]
        // a.w: beta sh as (kappa/2) beta; b.y and c.w (recD with F(Q))
        // carry (sin theta, cos theta) for the rotated odd seed
        ra = make_float4(p.th_hi, p.th_lo, p.kappa,
                         __fmul_rn(0.5f * p.kappa, beta));
        rb = make_float4(beta * p.ch, p.sth, beta, gam);
        const float fe = WITH_F ? -(p.r * p.r) : 0.f;
        rc = make_float4(dx, dy, dz, WITH_F ? fe : p.cth);
        re = make_float4(p.sigma2 * dx, p.sigma2 * dy, p.sigma2 * dz,
                         p.sigma2 * fe);
        if constexpr (WITH_F) recD[q] = p.cth;
      } else if constexpr (WITH_F) {
        recD[q] = 0.f;
      }
      recA[q] = ra;
      recB[q] = rb;
      recC[q] = rc;
      recE[q] = re;
    }
    if (has_next && tid < tN.y) sJb[jb ^ 1][tid] = pN;
    __syncthreads();
    auto pair_loop = [&](auto use_f) {
      constexpr bool UF = WITH_F && decltype(use_f)::value;
      for (int b = 0; b < tJ.y; ++b) {
        const int q = b * kTile + al;
        const float4 ra = recA[q];
        const float4 rb = recB[q];
        const float4 rc = recC[q];
        const float4 re = recE[q];
        float2 s, co;
        seed_sincos2r(kf, ra.x, ra.y, rb.y, WITH_F ? recD[q] : rc.w, s, co);
        float2 t = __fmul2_rn(f2(rb.z), s);
        float2 w = __ffma2_rn(co, f2(rb.x), __fmul2_rn(s, f2(ra.w)));
        float2 kg = make_float2(kf * rb.w, (kf + 1.0f) * rb.w);
        const float2 dkg = f2(2.0f * rb.w);
        const float2 kp = f2(ra.z), km = f2(-ra.z);
        const float2 dx2 = f2(rc.x), dy2 = f2(rc.y), dz2 = f2(rc.z);
        const float2 sx2 = f2(re.x), sy2 = f2(re.y), sz2 = f2(re.z);
        const float2 fe2 = f2(rc.w), fo2 = f2(re.w);
#pragma unroll
        for (int m = 0; m < M; ++m) {
          const float2 wn = __ffma2_rn(km, t, w);
          const float2 u = __fadd2_rn(w, wn);
          const float2 gk = __ffma2_rn(kg, u, t);
          if (m & 1) {
            ax[m] = __ffma2_rn(gk, sx2, ax[m]);
            ay[m] = __ffma2_rn(gk, sy2, ay[m]);
            az[m] = __ffma2_rn(gk, sz2, az[m]);
            if constexpr (UF) af[m] = __ffma2_rn(t, fo2, af[m]);
          } else {
            ax[m] = __ffma2_rn(gk, dx2, ax[m]);
            ay[m] = __ffma2_rn(gk, dy2, ay[m]);
            az[m] = __ffma2_rn(gk, dz2, az[m]);
            if constexpr (UF) af[m] = __ffma2_rn(t, fe2, af[m]);
          }
          t = __ffma2_rn(kp, wn, t);
          w = wn;
          kg = __fadd2_rn(kg, dkg);
        }
      }
    };
    const bool count_f = WITH_F && tj >= I;
    if (active) {
      if (count_f)
        pair_loop(BoolTag<true>());
      else
        pair_loop(BoolTag<false>());
    }
    if constexpr (WITH_F) {
      if (same) {
        flush_f(tJ.w, 0.5f);
      } else if (count_f) {
        f_sb = tJ.w;
        ++f_tiles;
      }
    }
  }
  if (cur_sb >= 0) flush(cur_sb, true);
  if constexpr (WITH_F) {
    if (f_tiles > 0) flush_f(f_sb, 1.f);
    __syncthreads();
    for (int i = tid; i < CPC * L; i += blockDim.x) {
      const int c = i / L;
      const int ch = blockIdx.y * CPC + c;
      const int k = kb0 + ch * L + i % L;
      if (ch < chunks_total && k < n_bins) {
        double sum = 0.0;
        for (int wp = 0; wp < CPC; ++wp)
          sum += (double)fsum[wp * CPC * L + i] - (double)fcmp[wp * CPC * L + i];
        fpart[(size_t)I * n_bins + k] = sum;
      }
    }
  }
}

template <int L, int CPC, int MINB>
__global__ void __launch_bounds__(kTile * CPC, MINB)
    gradfq2_kernel(const float *__restrict__ pos, const int *__restrict__ perm,
                   const int4 *__restrict__ tiles,
                   const int2 *__restrict__ cfg_tiles, float dq_hi,
                   float dq_lo, int kb0, int chunks_total, int n_bins,
                   const float *__restrict__ coef, int n_species,
                   float *__restrict__ out, JSplit js) {
  gradfq2_body<L, CPC, false>(pos, perm, tiles, cfg_tiles, dq_hi, dq_lo, kb0,
                              chunks_total, n_bins, coef, n_species, out,
                              nullptr, nullptr, 0, js);
}

// F(Q) pair sums and dF/dx in one pass (see gradfq2_body).  Dynamic shared
// memory: 3 kTile^2 float4 records + 2 CPC * CPC * L floats + kTile^2
// floats (cos theta).
template <int L, int CPC, int MINB>
__global__ void __launch_bounds__(kTile * CPC, MINB)
    fqgrad2_kernel(const float *__restrict__ pos, const int *__restrict__ perm,
                   const int4 *__restrict__ tiles,
                   const int2 *__restrict__ cfg_tiles, float dq_hi,
                   float dq_lo, int kb0, int chunks_total, int n_bins,
                   const float *__restrict__ coef, int n_species,
                   float *__restrict__ out, const float *__restrict__ ftab,
                   double *__restrict__ fpart, int tile0, JSplit js) {
  gradfq2_body<L, CPC, true>(pos, perm, tiles, cfg_tiles, dq_hi, dq_lo, kb0,
                             chunks_total, n_bins, coef, n_species, out, ftab,
                             fpart, tile0, js);
}

// F(Q) of the fused pass: S_k = sum over the tiles [t0, t1) of the
// configuration of fpart[tile][k] (fixed order), F_k as fq_finish_kernel.
// With sums != nullptr the raw S_k (0 below kb_out) go there instead (one
// part of a configuration split across processes; pyiid_fq_from_sums
// finishes the summed parts).
// One warp per bin: lanes take rows t0 + lane, t0 + lane + 32, ... and the
// warp adds the lane sums in a fixed shuffle order (bitwise reproducible).
__global__ void fqgrad_finish_kernel(const double *__restrict__ fpart,
                                     int t0, int t1, const double *__restrict__ na,
                                     int n_bins, int kb_out,
                                     float *__restrict__ fq,
                                     double *__restrict__ sums) {
  const int k = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (k >= n_bins) return;  // whole warps leave together
  double s = 0.0;
  if (k >= kb_out)
    for (int t = t0 + lane; t < t1; t += 32) s += fpart[(size_t)t * n_bins + k];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane) return;
  if (sums) {
    sums[k] = s;
  } else {
    fq[k] = (k >= kb_out) ? fq_value(s, na[k]) : 0.f;
  }
}

// grad[i] = nan_to_num(sum over parts p of parts[p * stride + i]) for bins
// k >= kbo, 0 below: the J-split parts of gradfq2_body added in part order.
// Four elements per thread when n_bins % 4 == 0 and both pointers are
// 16-byte aligned (the caller's gradient may be any float array), else one.
__device__ __forceinline__ float nan_to_num_f(float v) {
  return isnan(v) ? 0.f : (isinf(v) ? copysignf(3.402823466e38f, v) : v);
}

__global__ void combine_grad_parts_kernel(const float *__restrict__ parts,
                                          int n_parts, size_t stride,
                                          size_t n, int n_bins, int kbo,
                                          float *__restrict__ grad) {
  const size_t t0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t nt = (size_t)gridDim.x * blockDim.x;
  const bool aligned = ((reinterpret_cast<uintptr_t>(parts) |
                         reinterpret_cast<uintptr_t>(grad)) & 15) == 0;
  if (n_bins % 4 == 0 && aligned && n_parts <= kMaxJSplit) {
    const float4 *p4 = reinterpret_cast<const float4 *>(parts);
    float4 *g4 = reinterpret_cast<float4 *>(grad);
    for (size_t i = t0; i < n / 4; i += nt) {
      // every part's load in flight before the fixed-order sum (n_parts is
      // at most kMaxJSplit)
      float4 a[kMaxJSplit];
#pragma unroll
      for (int p = 0; p < kMaxJSplit; ++p)
        if (p < n_parts) a[p] = p4[p * (stride / 4) + i];
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int p = 0; p < kMaxJSplit; ++p) {
        if (p < n_parts) {
          v.x += a[p].x;
          v.y += a[p].y;
          v.z += a[p].z;
          v.w += a[p].w;
        }
      }
      const int k = (int)((4 * i) % n_bins);
      v.x = k >= kbo ? nan_to_num_f(v.x) : 0.f;
      v.y = k + 1 >= kbo ? nan_to_num_f(v.y) : 0.f;
      v.z = k + 2 >= kbo ? nan_to_num_f(v.z) : 0.f;
      v.w = k + 3 >= kbo ? nan_to_num_f(v.w) : 0.f;
      g4[i] = v;
    }
    return;
  }
  for (size_t i = t0; i < n; i += nt) {
    float v = 0.f;
    if ((int)(i % n_bins) >= kbo) {
      for (int p = 0; p < n_parts; ++p) v += parts[p * stride + i];
      v = nan_to_num_f(v);
    }
    grad[i] = v;
  }
}

// F_k = 2 nan_to_num(S_k / na_k) for k >= kb_out (0 below) from summed raw
// sums (the finishing step of a configuration split across processes).
__global__ void fq_from_sums_kernel(const double *__restrict__ sums,
                                    const double *__restrict__ na, int n_bins,
                                    int kb_out, float *__restrict__ fq) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_bins) return;
  fq[k] = (k >= kb_out) ? fq_value(sums[k], na[k]) : 0.f;
}

// Zeroes bins [0, kb) of the gradient rows of the atoms of tiles [t0, t1).
__global__ void zero_low_bins_kernel(const int *__restrict__ perm,
                                     const int4 *__restrict__ tiles, int t0,
                                     int kb, int n_bins,
                                     float *__restrict__ grad) {
  const int4 t = tiles[t0 + blockIdx.x];
  for (int i = threadIdx.x; i < t.y * 3 * kb; i += blockDim.x) {
    const int a = i / (3 * kb), rest = i % (3 * kb);
    const int c = rest / kb, k = rest % kb;
    grad[((size_t)perm[t.x + a] * 3 + c) * n_bins + k] = 0.f;
  }
}

// =================================================================== adjoint
// Exact position gradient of Rw or chi^2 (get_grad_rw / get_grad_chi_sq,
// kernels/master_kernel.py:293-376, with get_grad_scale :392-396), which the
// reference forms as a contraction of the [N, 3, R] grad_pdf array; both are
// linear in dG, so the contraction moves back through G = T F to the bins:
// d(potential)/dx_a = sum_b (x_a - x_b) s_ab,  s_ab = sum_k W^{sa sb}_k g_k(r_ab)
// with W_k = 2 w_k f_sa f_sb / na_k and w = T c the back-projected G(r)
// adjoint.  Owner-computes: CTA = tile I, thread (atom a = lane, group =
// warp); group gp handles b = gp, gp + 8, ... of every tile J, so the lanes of
// a warp share b and every table read is a broadcast of one address.
// Packed even/odd recurrence (pair_math.cuh), re-seeded every RS bins from
// kb0 (RS a multiple of 4); the last block runs only up to the last bin.
// Tables hold, for every bin pair (kk, kk+1), kk = k - kb0 even,
//   (A_kk, A_kk+1, B_kk, B_kk+1),  A_k = k W_k, B_k = W_k,
// and the sign sigma2^m of step m is applied by accumulating even and odd
// steps separately, so with t, w scaled by beta = -1/r^3 and
// gamma' = -r dq/(2 ch):
//   s_ab = gamma' (Ae + sigma2 Ao) + (Be + sigma2 Bo),
//   Ae = sum_{m even} A (w_m + w_{m+1}),  Be = sum_{m even} B t_m, ...
// Per two bins and ordered pair: 5 packed FP32x2 instructions + 1 LDS.128.
template <int RS>
__global__ void __launch_bounds__(kBlock)
    adjoint_kernel(const float *__restrict__ pos, const int *__restrict__ perm,
                   const int4 *__restrict__ tiles,
                   const int2 *__restrict__ cfg_tiles, float dq_hi,
                   float dq_lo, int kb0, int kp,
                   const float4 *__restrict__ tabs, int n_species,
                   float *__restrict__ grad) {
  static_assert(RS % 4 == 0, "RS must be a multiple of 4");
  extern __shared__ float4 stab[];  // [n_species][kp/2]
  __shared__ float4 sI[kTile], sJ[kTile];
  __shared__ float sred[kBlock / kTile][kTile][3];

  const int4 ti = tiles[blockIdx.x];
  const int2 ct = cfg_tiles[ti.z];
  const int tid = threadIdx.x;
  const int lane = tid % kTile;
  const int grp = tid / kTile;
  const int ngrp = blockDim.x / kTile;
  const int kh = kp / 2;  // packed steps (bin pairs) in the table

  const float4 *src = tabs + ((size_t)ti.z * n_species + ti.w) * n_species * kh;
  for (int i = tid; i < n_species * kh; i += blockDim.x) stab[i] = src[i];
  if (tid < ti.y) sI[tid] = load_atom(pos, perm, ti.x + tid);

  float gx = 0.f, gy = 0.f, gz = 0.f;
  for (int tj = ct.x; tj < ct.y; ++tj) {
    const int4 tJ = tiles[tj];
    __syncthreads();
    if (tid < tJ.y) sJ[tid] = load_atom(pos, perm, tJ.x + tid);
    __syncthreads();
    const bool same = (tj == (int)blockIdx.x);
    const float4 *tab = stab + (size_t)tJ.w * kh;
    if (lane < ti.y) {
      const float4 pa = sI[lane];
      for (int b = grp; b < tJ.y; b += ngrp) {
        if (same && b == lane) continue;
        const float4 pb = sJ[b];
        float dx, dy, dz;
        PairPhase2 p = pair_phase2(pa.x, pa.y, pa.z, pb.x, pb.y, pb.z, dq_hi,
                                   dq_lo, dx, dy, dz);
        const float beta = -(p.inv_r * p.inv_r * p.inv_r);
        const float2 c1 = f2(beta * p.ch), c2 = f2(beta * p.sh);
        const float gam = __fdividef(-p.r * dq_hi, 2.0f * p.ch);  // 2ch in [1.41, 2]
        const float2 kpos = f2(p.kappa), kneg = f2(-p.kappa);
        float2 ae = f2(0.f), ao = f2(0.f), be = f2(0.f), bo = f2(0.f);
        for (int blk = 0; blk < kh; blk += RS / 2) {
          float2 s, co;
          seed_sincos2r((float)(kb0 + 2 * blk), p.th_hi, p.th_lo, p.sth,
                        p.cth, s, co);
          float2 t = __fmul2_rn(f2(beta), s);
          float2 w = __ffma2_rn(co, c1, __fmul2_rn(s, c2));
          const float4 *tb = tab + blk;
          if (blk + RS / 2 <= kh) {
#pragma unroll
            for (int m = 0; m < RS / 2; m += 2) {
              float4 wt = tb[m];
              float2 wn = __ffma2_rn(kneg, t, w);
              ae = __ffma2_rn(make_float2(wt.x, wt.y), __fadd2_rn(w, wn), ae);
              be = __ffma2_rn(make_float2(wt.z, wt.w), t, be);
              t = __ffma2_rn(kpos, wn, t);
              w = wn;
              wt = tb[m + 1];
              wn = __ffma2_rn(kneg, t, w);
              ao = __ffma2_rn(make_float2(wt.x, wt.y), __fadd2_rn(w, wn), ao);
              bo = __ffma2_rn(make_float2(wt.z, wt.w), t, bo);
              t = __ffma2_rn(kpos, wn, t);
              w = wn;
            }
          } else {
            const int nm = kh - blk;  // even: kp is a multiple of 4
            for (int m = 0; m < nm; m += 2) {
              float4 wt = tb[m];
              float2 wn = __ffma2_rn(kneg, t, w);
              ae = __ffma2_rn(make_float2(wt.x, wt.y), __fadd2_rn(w, wn), ae);
              be = __ffma2_rn(make_float2(wt.z, wt.w), t, be);
              t = __ffma2_rn(kpos, wn, t);
              w = wn;
              wt = tb[m + 1];
              wn = __ffma2_rn(kneg, t, w);
              ao = __ffma2_rn(make_float2(wt.x, wt.y), __fadd2_rn(w, wn), ao);
              bo = __ffma2_rn(make_float2(wt.z, wt.w), t, bo);
              t = __ffma2_rn(kpos, wn, t);
              w = wn;
            }
          }
        }
        const float sg = p.sigma2;
        const float A = (ae.x + ae.y) + sg * (ao.x + ao.y);
        const float B = (be.x + be.y) + sg * (bo.x + bo.y);
        const float sab = fmaf(gam, A, B);
        gx = fmaf(sab, dx, gx);
        gy = fmaf(sab, dy, gy);
        gz = fmaf(sab, dz, gz);
      }
    }
  }
  sred[grp][lane][0] = gx;
  sred[grp][lane][1] = gy;
  sred[grp][lane][2] = gz;
  __syncthreads();
  if (tid < ti.y * 3) {
    const int a = tid / 3, cpt = tid % 3;
    float sum = 0.f;
    for (int gg = 0; gg < ngrp; ++gg) sum += sred[gg][a][cpt];
    grad[(size_t)perm[ti.x + a] * 3 + cpt] = sum;
  }
}

// ======================================================= symmetric adjoint
// Each unordered pair once.  CTA = F(Q) work item (tile I, tiles [J0, J1) with
// J <= I); lane a of tile I, warp (group) gp handles b = gp, gp + 8, ... of
// each tile J (for the diagonal tile only b < a).  The i-side
// s_ab (x_a - x_b) accumulates in the lane's registers; the j-side
// -s_ab (x_a - x_b) of atom b is summed over the warp's 32 lanes with
// shuffles and kept in shared memory per (J, b).  Each CTA writes its i-side
// rows [32][3] at part[ioff[item]] and its j-side rows [(J1-J0)*32][3] at
// part[joff[item]]; adjoint_reduce_kernel adds them per atom in a fixed
// order (bitwise reproducible).  Table layout and recurrence as in
// adjoint_kernel.
template <int RS>
__global__ void __launch_bounds__(kBlock)
    adjoint_sym_kernel(const float *__restrict__ pos,
                       const int *__restrict__ perm,
                       const int4 *__restrict__ tiles,
                       const int4 *__restrict__ items,
                       const int *__restrict__ order, float dq_hi,
                       float dq_lo, int kb0, int kp,
                       const float4 *__restrict__ tabs, int n_species,
                       const int *__restrict__ ioff,
                       const int *__restrict__ joff,
                       float *__restrict__ part) {
  static_assert(RS % 4 == 0, "RS must be a multiple of 4");
  extern __shared__ float4 stab[];  // [kp/2] for this item's species pair
  __shared__ float4 sI[kTile], sJ[kTile];
  __shared__ float sred[kBlock / kTile][kTile][3];
  __shared__ float sjac[kJMaxTiles][kTile][3];

  const int item = order ? order[blockIdx.x] : (int)blockIdx.x;
  const int4 it = items[item];
  const int4 ti = tiles[it.x];
  const int tid = threadIdx.x;
  const int lane = tid % kTile;
  const int grp = tid / kTile;
  const int ngrp = blockDim.x / kTile;
  const int kh = kp / 2;
  const int sa = ti.w;
  const int sbs = tiles[it.y].w;  // every tile of the item has this species

  const float4 *src =
      tabs + (((size_t)ti.z * n_species + sa) * n_species + sbs) * kh;
  for (int i = tid; i < kh; i += blockDim.x) stab[i] = src[i];
  if (tid < ti.y) sI[tid] = load_atom(pos, perm, ti.x + tid);
  for (int i = tid; i < (it.z - it.y) * kTile * 3; i += blockDim.x)
    (&sjac[0][0][0])[i] = 0.f;

  float gx = 0.f, gy = 0.f, gz = 0.f;
  for (int tj = it.y; tj < it.z; ++tj) {
    const int4 tJ = tiles[tj];
    const int jl = tj - it.y;
    __syncthreads();
    if (tid < tJ.y) sJ[tid] = load_atom(pos, perm, tJ.x + tid);
    __syncthreads();
    const bool diag = (tj == it.x);
    const float4 pa = sI[lane < ti.y ? lane : 0];
    for (int b = grp; b < tJ.y; b += ngrp) {
      const bool valid = (lane < ti.y) && (!diag || b < lane);
      float jx = 0.f, jy = 0.f, jz = 0.f;
      if (valid) {
        const float4 pb = sJ[b];
        float dx, dy, dz;
        PairPhase2 p = pair_phase2(pa.x, pa.y, pa.z, pb.x, pb.y, pb.z, dq_hi,
                                   dq_lo, dx, dy, dz);
        const float beta = -(p.inv_r * p.inv_r * p.inv_r);
        const float2 c1 = f2(beta * p.ch), c2 = f2(beta * p.sh);
        const float gam = __fdividef(-p.r * dq_hi, 2.0f * p.ch);  // 2ch in [1.41, 2]
        const float2 kpos = f2(p.kappa), kneg = f2(-p.kappa);
        float2 ae = f2(0.f), ao = f2(0.f), be = f2(0.f), bo = f2(0.f);
        for (int blk = 0; blk < kh; blk += RS / 2) {
          float2 s, co;
          seed_sincos2r((float)(kb0 + 2 * blk), p.th_hi, p.th_lo, p.sth,
                        p.cth, s, co);
          float2 t = __fmul2_rn(f2(beta), s);
          float2 w = __ffma2_rn(co, c1, __fmul2_rn(s, c2));
          const float4 *tb = stab + blk;
          if (blk + RS / 2 <= kh) {
#pragma unroll
            for (int m = 0; m < RS / 2; m += 2) {
              float4 wt = tb[m];
              float2 wn = __ffma2_rn(kneg, t, w);
              ae = __ffma2_rn(make_float2(wt.x, wt.y), __fadd2_rn(w, wn), ae);
              be = __ffma2_rn(make_float2(wt.z, wt.w), t, be);
              t = __ffma2_rn(kpos, wn, t);
              w = wn;
              wt = tb[m + 1];
              wn = __ffma2_rn(kneg, t, w);
              ao = __ffma2_rn(make_float2(wt.x, wt.y), __fadd2_rn(w, wn), ao);
              bo = __ffma2_rn(make_float2(wt.z, wt.w), t, bo);
              t = __ffma2_rn(kpos, wn, t);
              w = wn;
            }
          } else {
            const int nm = kh - blk;
            for (int m = 0; m < nm; m += 2) {
              float4 wt = tb[m];
              float2 wn = __ffma2_rn(kneg, t, w);
              ae = __ffma2_rn(make_float2(wt.x, wt.y), __fadd2_rn(w, wn), ae);
              be = __ffma2_rn(make_float2(wt.z, wt.w), t, be);
              t = __ffma2_rn(kpos, wn, t);
              w = wn;
              wt = tb[m + 1];
              wn = __ffma2_rn(kneg, t, w);
              ao = __ffma2_rn(make_float2(wt.x, wt.y), __fadd2_rn(w, wn), ao);
              bo = __ffma2_rn(make_float2(wt.z, wt.w), t, bo);
              t = __ffma2_rn(kpos, wn, t);
              w = wn;
            }
          }
        }
        const float sg = p.sigma2;
        const float A = (ae.x + ae.y) + sg * (ao.x + ao.y);
        const float B = (be.x + be.y) + sg * (bo.x + bo.y);
        const float sab = fmaf(gam, A, B);
        gx = fmaf(sab, dx, gx);
        gy = fmaf(sab, dy, gy);
        gz = fmaf(sab, dz, gz);
        jx = -sab * dx;
        jy = -sab * dy;
        jz = -sab * dz;
      }
      // j-side: sum over the warp's lanes (all 32 lanes take part)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        jx += __shfl_xor_sync(0xffffffffu, jx, o);
        jy += __shfl_xor_sync(0xffffffffu, jy, o);
        jz += __shfl_xor_sync(0xffffffffu, jz, o);
      }
      if (lane == 0) {
        sjac[jl][b][0] += jx;
        sjac[jl][b][1] += jy;
        sjac[jl][b][2] += jz;
      }
    }
  }
  sred[grp][lane][0] = gx;
  sred[grp][lane][1] = gy;
  sred[grp][lane][2] = gz;
  __syncthreads();
  float *pi = part + ioff[item];
  for (int i = tid; i < kTile * 3; i += blockDim.x) {
    const int a = i / 3, c = i % 3;
    float sum = 0.f;
    for (int gg = 0; gg < ngrp; ++gg) sum += sred[gg][a][c];
    pi[i] = sum;
  }
  float *pj = part + joff[item];
  for (int i = tid; i < (it.z - it.y) * kTile * 3; i += blockDim.x)
    pj[i] = (&sjac[0][0][0])[i];
}

// grad[perm[t.start + a]][c] = sum of the partial rows listed for tile t
// (CSR: entries tile_ptr[t] .. tile_ptr[t+1]-1 are float offsets of
// [32][3] blocks), in list order.
__global__ void adjoint_reduce_kernel(const float *__restrict__ part,
                                      const int *__restrict__ tile_ptr,
                                      const int *__restrict__ entries,
                                      const int4 *__restrict__ tiles,
                                      const int *__restrict__ perm,
                                      int n_tiles, float *__restrict__ grad) {
  const int t = blockIdx.x;
  if (t >= n_tiles) return;
  const int4 ti = tiles[t];
  const int i = threadIdx.x;  // 0 .. 95
  if (i >= ti.y * 3) return;
  float s = 0.f;
  for (int e = tile_ptr[t]; e < tile_ptr[t + 1]; ++e) s += part[entries[e] + i];
  grad[(size_t)perm[ti.x + i / 3] * 3 + i % 3] = s;
}

}  // namespace pyiid
