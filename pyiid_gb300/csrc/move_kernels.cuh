// move_kernels.cuh -- single-atom Metropolis moves with O(N K) exact energy
// changes.
//
// Moving atom a from x to x' changes only the N-1 pair terms that involve a:
//   S'_k = S_k + f_sa(Q_k) sum_{j != a} f_sj(Q_k) [w(|x' - x_j|) - w(|x - x_j|)],
//   w(r) = sin(Q_k r) / r,
// so a proposal costs 2 (N-1) K sinusoid terms instead of N(N-1)/2 K.  The
// raw Debye sums S_k of every chain are kept on the device in FP64; a step is
//   move_delta_kernel  (pair terms of the moved atom, old and new position)
//   move_fq_kernel     (F'_k = 2 nan_to_num(float(S_k + dS_k) / float(na_k)))
//   pdf_kernel         (G'(r) = sum_k F'_k T[k][r])
//   mh_accept_kernel   (potential of G', Metropolis test, state update)
// with no host round trip, so any number of steps can be enqueued at once or
// captured in a CUDA graph.  Proposals come from a counter-based generator
// (Philox4x32-10) keyed by the caller's seed and counted per chain, so a run
// is reproducible and independent of how steps are batched into calls.
#pragma once

#include "debye_kernels.cuh"
#include "transform_kernels.cuh"

namespace pyiid {

constexpr int kMoveTiles = 4;  // tiles (all of one species) per work item
constexpr int kMoveL = 32;     // bins per thread between re-seeds

// Philox4x32 with 10 rounds: Salmon, Moraes, Dror and Shaw, "Parallel random
// numbers: as easy as 1, 2, 3", SC 2011.  Round multipliers and Weyl key
// increments as published there.
__host__ __device__ inline uint4 philox4x32_10(uint4 c, uint32_t k0,
                                               uint32_t k1) {
  for (int i = 0; i < 10; ++i) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c.x;
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c.z;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

// One proposal: the atom (index within its configuration, caller order), its
// displacement and log(u) of the acceptance uniform.
struct MoveProposal {
  int atom;
  float d[3];
  double logu;
};

// float in (0, 1): 23 random bits, centred (exact in float)
__device__ __forceinline__ float unit_float(uint32_t x) {
  return (float)(2u * (x >> 9) + 1u) * 5.9604644775390625e-08f;  // 2^-24
}

// Proposal number `step` of chain `chain`:
//   counter words (step lo, step hi, chain, 0/1), key (seed lo, seed hi);
//   atom  = floor(r0.x * n / 2^32)
//   d     = sigma * (n0, n1, n2), Box-Muller on (r0.y, r0.z) and (r0.w, r1.x)
//   log u = log((53-bit integer of r1.y, r1.z + 1/2) / 2^53)
__device__ __forceinline__ MoveProposal make_proposal(uint32_t seed_lo,
                                                      uint32_t seed_hi,
                                                      unsigned long long step,
                                                      int chain, int n,
                                                      float sigma) {
  const uint32_t slo = (uint32_t)step, shi = (uint32_t)(step >> 32);
  const uint4 r0 =
      philox4x32_10(make_uint4(slo, shi, (uint32_t)chain, 0u), seed_lo, seed_hi);
  const uint4 r1 =
      philox4x32_10(make_uint4(slo, shi, (uint32_t)chain, 1u), seed_lo, seed_hi);
  MoveProposal p;
  p.atom = (int)(((uint64_t)r0.x * (uint64_t)(n > 0 ? n : 0)) >> 32);
  float s, c;
  const float ra = sqrtf(-2.0f * logf(unit_float(r0.y)));
  sincospif(2.0f * unit_float(r0.z), &s, &c);
  p.d[0] = sigma * (ra * c);
  p.d[1] = sigma * (ra * s);
  const float rb = sqrtf(-2.0f * logf(unit_float(r0.w)));
  sincospif(2.0f * unit_float(r1.x), &s, &c);
  p.d[2] = sigma * (rb * c);
  const uint64_t m = ((((uint64_t)r1.y) << 32) | r1.z) >> 11;
  p.logu = log(((double)m + 0.5) * 1.1102230246251565e-16);  // 2^-53
  return p;
}

// Pair terms of the moved atom.  One CTA per work item (chain, species,
// tiles [t0, t1) of that species: consecutive sorted atoms) and bin block;
// thread (chunk c, group g) accumulates bins [kbase, kbase + L) of
//   sum_j w(|x' - x_j|) - w(|x - x_j|)
// over the atoms j = g, g + n_groups, ... of the item, with the packed
// even/odd recurrence of pair_math.cuh for both sinusoids.  The groups are
// reduced through shared memory in FP64 and the CTA writes one partial row.
// The moved atom itself contributes nothing (its records are zero).
// Dynamic shared memory: 4 * kMoveTiles * 32 float4 records +
// n_groups * n_chunks * L floats.
__global__ void __launch_bounds__(kBlock)
    move_delta_kernel(const float *__restrict__ pos,
                      const int *__restrict__ perm,
                      const int4 *__restrict__ tiles,
                      const int4 *__restrict__ mitems,
                      const int *__restrict__ mitem_begin,
                      const int *__restrict__ offsets,
                      const unsigned long long *__restrict__ counter,
                      uint32_t seed_lo, uint32_t seed_hi, float sigma,
                      float dq_hi, float dq_lo, int kb0, int n_chunks,
                      int n_groups, int n_bins,
                      MoveProposal *__restrict__ prop_out,
                      double *__restrict__ partial) {
  constexpr int L = kMoveL;
  constexpr int M = L / 2;
  constexpr int NJ = kMoveTiles * kTile;
  extern __shared__ float4 smem[];
  float4 *oA = smem;
  float4 *oB = oA + NJ;
  float4 *nA = oB + NJ;
  float4 *nB = nA + NJ;
  float *red = reinterpret_cast<float *>(nB + NJ);
  __shared__ float sx[6];
  __shared__ int s_atom;

  const int4 it = mitems[blockIdx.x];  // (chain, species, t0, t1)
  const int chain = it.x;
  const int tid = threadIdx.x;
  if (tid == 0) {
    const int base = offsets[chain];
    const int n = offsets[chain + 1] - base;
    const MoveProposal p =
        make_proposal(seed_lo, seed_hi, counter[chain], chain, n, sigma);
    if (blockIdx.y == 0 && (int)blockIdx.x == mitem_begin[chain])
      prop_out[chain] = p;
    const int a = base + p.atom;  // items exist only for n >= 1
    s_atom = a;
    const float x = pos[3 * a], y = pos[3 * a + 1], z = pos[3 * a + 2];
    sx[0] = x;
    sx[1] = y;
    sx[2] = z;
    sx[3] = __fadd_rn(x, p.d[0]);
    sx[4] = __fadd_rn(y, p.d[1]);
    sx[5] = __fadd_rn(z, p.d[2]);
  }
  __syncthreads();
  const int s0 = tiles[it.z].x;
  const int4 tl = tiles[it.w - 1];
  const int nj = tl.x + tl.y - s0;
  const int a = s_atom;
  for (int q = tid; q < nj; q += blockDim.x) {
    const int o = perm[s0 + q];
    if (o == a) {
      oA[q] = nA[q] = make_float4(0.f, 0.f, 0.f, 1.f);
      oB[q] = nB[q] = make_float4(0.f, 0.f, 0.f, 0.f);
    } else {
      const float xj = pos[3 * o], yj = pos[3 * o + 1], zj = pos[3 * o + 2];
      float dx, dy, dz;
      const PairPhase2 po =
          pair_phase2(sx[0], sx[1], sx[2], xj, yj, zj, dq_hi, dq_lo, dx, dy, dz);
      oA[q] = make_float4(po.th_hi, po.th_lo, po.kappa, po.sigma2);
      oB[q] = make_float4(po.ch * po.inv_r, po.sh * po.inv_r, po.inv_r, 0.f);
      const PairPhase2 pn =
          pair_phase2(sx[3], sx[4], sx[5], xj, yj, zj, dq_hi, dq_lo, dx, dy, dz);
      nA[q] = make_float4(pn.th_hi, pn.th_lo, pn.kappa, pn.sigma2);
      nB[q] = make_float4(pn.ch * pn.inv_r, pn.sh * pn.inv_r, pn.inv_r, 0.f);
    }
  }
  __syncthreads();

  const int c = tid % n_chunks;
  const int g = tid / n_chunks;
  const int kbase = kb0 + (blockIdx.y * n_chunks + c) * L;
  const float kf = (float)kbase;
  float2 acc[M];
#pragma unroll
  for (int m = 0; m < M; ++m) acc[m] = f2(0.f);
  if (g < n_groups) {
    for (int q = g; q < nj; q += n_groups) {
      float4 ra = nA[q], rb = nB[q];
      float2 s, co;
      seed_sincos2(kf, ra.x, ra.y, s, co);
      float2 tn = __fmul2_rn(f2(rb.z), s);
      float2 wn = __ffma2_rn(co, f2(rb.x), __fmul2_rn(s, f2(rb.y)));
      const float2 kpn = f2(ra.z), kmn = f2(-ra.z), sgn = f2(ra.w);
      ra = oA[q];
      rb = oB[q];
      seed_sincos2(kf, ra.x, ra.y, s, co);
      float2 to = __fmul2_rn(f2(rb.z), s);
      float2 wo = __ffma2_rn(co, f2(rb.x), __fmul2_rn(s, f2(rb.y)));
      const float2 kpo = f2(ra.z), kmo = f2(-ra.z), sgo = f2(-ra.w);
#pragma unroll
      for (int m = 0; m < M; ++m) {
        if (m & 1) {
          acc[m] = __ffma2_rn(tn, sgn, acc[m]);
          acc[m] = __ffma2_rn(to, sgo, acc[m]);
        } else {
          acc[m] = __fadd2_rn(acc[m], tn);
          acc[m] = __ffma2_rn(to, f2(-1.f), acc[m]);
        }
        if (m + 1 < M) {
          wn = __ffma2_rn(kmn, tn, wn);
          tn = __ffma2_rn(kpn, wn, tn);
          wo = __ffma2_rn(kmo, to, wo);
          to = __ffma2_rn(kpo, wo, to);
        }
      }
    }
    const int nk = n_chunks * L;
#pragma unroll
    for (int m = 0; m < M; ++m) {
      red[g * nk + c * L + 2 * m] = acc[m].x;
      red[g * nk + c * L + 2 * m + 1] = acc[m].y;
    }
  }
  __syncthreads();
  const int nk = n_chunks * L;
  const int kfirst = kb0 + blockIdx.y * nk;
  double *out = partial + (size_t)blockIdx.x * n_bins;
  for (int i = tid; i < nk; i += blockDim.x) {
    const int k = kfirst + i;
    if (k >= n_bins) continue;
    double s = 0.0;
    for (int gg = 0; gg < n_groups; ++gg) s += (double)red[gg * nk + i];
    out[k] = s;
  }
}

// Proposed F' of every chain:
//   dS_k = f_sa(Q_k) sum_{items of the chain} f_s(item)(Q_k) partial[item][k]
//   F'_k = 2 nan_to_num(float(S_k + dS_k) / float(na_k))  for k >= kmin, else 0.
// grid (ceil(n_bins / 128), n_chains)
__global__ void move_fq_kernel(const double *__restrict__ partial,
                               const int4 *__restrict__ mitems,
                               const int *__restrict__ mitem_begin,
                               const int *__restrict__ offsets,
                               const int *__restrict__ species,
                               const MoveProposal *__restrict__ prop,
                               const float *__restrict__ ftab,
                               const double *__restrict__ na,
                               const double *__restrict__ sraw, int n_bins,
                               int kmin, float *__restrict__ fq_prop,
                               double *__restrict__ ds_out) {
  const int b = blockIdx.y;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_bins) return;
  const int base = offsets[b];
  const int n = offsets[b + 1] - base;
  double ds = 0.0;
  float f = 0.f;
  if (n >= 2 && k >= kmin) {
    const int sa = species[base + prop[b].atom];
    double d = 0.0;
    for (int i = mitem_begin[b]; i < mitem_begin[b + 1]; ++i)
      d += (double)ftab[mitems[i].y * n_bins + k] *
           partial[(size_t)i * n_bins + k];
    ds = (double)ftab[sa * n_bins + k] * d;
    const size_t bk = (size_t)b * n_bins + k;
    f = fq_value(sraw[bk] + ds, na[bk]);
  }
  fq_prop[(size_t)b * n_bins + k] = f;
  ds_out[(size_t)b * n_bins + k] = ds;
}

// Metropolis test and state update, one CTA per chain: the potential of the
// proposed G'(r), accept when log u < -conv (V' - V) / kT (never for a NaN
// potential), then on acceptance move the atom, add dS to S and store V'.
// The chain's proposal counter advances either way.  Chains with fewer than
// two atoms have no pair terms and never move.
// trace (optional) [n_chains][8]: atom, x', y', z', log u, V', accepted, V.
__global__ void mh_accept_kernel(
    float *__restrict__ pos, const int *__restrict__ offsets,
    const MoveProposal *__restrict__ prop, const double *__restrict__ gobs,
    const double *__restrict__ gcalc, int n_r, int potential, double conv,
    double kT, const double *__restrict__ ds, double *__restrict__ sraw,
    int n_bins, double *__restrict__ energy,
    unsigned long long *__restrict__ counter,
    long long *__restrict__ accepted, double *__restrict__ trace) {
  __shared__ double scratch[32 * 3];
  const int b = blockIdx.x;
  const int base = offsets[b];
  const int n = offsets[b + 1] - base;
  if (n < 2) {
    if (threadIdx.x == 0) {
      counter[b] += 1ull;
      if (trace)
        for (int i = 0; i < 8; ++i) trace[(size_t)b * 8 + i] = 0.0;
    }
    return;
  }
  const PotentialValue pv = potential_value(gobs, gcalc + (size_t)b * n_r,
                                            n_r, potential, scratch);
  const MoveProposal p = prop[b];
  const double e0 = energy[2 * b];
  const bool acc = p.logu < -conv * (pv.value - e0) / kT;
  if (acc)
    for (int k = threadIdx.x; k < n_bins; k += blockDim.x)
      sraw[(size_t)b * n_bins + k] += ds[(size_t)b * n_bins + k];
  if (threadIdx.x == 0) {
    const int a = base + p.atom;
    float xn[3];
    for (int i = 0; i < 3; ++i) xn[i] = __fadd_rn(pos[3 * a + i], p.d[i]);
    if (acc) {
      for (int i = 0; i < 3; ++i) pos[3 * a + i] = xn[i];
      energy[2 * b] = pv.value;
      energy[2 * b + 1] = pv.scale;
      accepted[b] += 1;
    }
    if (trace) {
      double *t = trace + (size_t)b * 8;
      t[0] = (double)p.atom;
      t[1] = xn[0];
      t[2] = xn[1];
      t[3] = xn[2];
      t[4] = p.logu;
      t[5] = pv.value;
      t[6] = acc ? 1.0 : 0.0;
      t[7] = e0;
    }
    counter[b] += 1ull;
  }
}

}  // namespace pyiid
