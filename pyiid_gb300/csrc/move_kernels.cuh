// move_kernels.cuh -- single-atom Metropolis moves with O(N K) exact energy
// changes.
//
// Moving atom a from x to x' changes only the N-1 pair terms that involve a:
//   S'_k = S_k + f_sa(Q_k) sum_{j != a} f_sj(Q_k) [w(|x' - x_j|) - w(|x - x_j|)],
//   w(r) = sin(Q_k r) / r,
// so a proposal costs 2 (N-1) K sinusoid terms instead of N(N-1)/2 K.  (The
// reference re-evaluates the whole configuration for every Monte Carlo
// move: add_atom / del_atom in pyiid/sim/gcmc.py:13-114; its acceptance
// rules are mh_accept, pyiid/sim/hmc.py:66-92, and the grand-canonical
// rule of gcmc.py:13-114.)
//
// The potential needs G only through three scalars.  With G = T^T F (the
// transform of the reference as a K x R matrix T), v = T gobs and the Gram
// matrix M = T T^T (K x K, symmetric):
//   G.gobs = F.v = u,   G.G = F^T M F = q,   |gobs - s G|^2 = gobs.gobs - 2 s u + s^2 q.
// Each chain keeps S (FP64), F (the float F the reference transforms), u, q
// and ee = |gobs - s G|^2 at the optimal scale s = u / q; a proposal
// F' = F + dF gives
//   du = dF.v,   dq = dF^T M (F + F'),
//   ee' - ee = -[(2 u du + du^2) q - u^2 dq] / (q (q + dq)),
// which costs K^2 instead of K R per chain and is accurate in FP32 because
// only small increments are formed (no cancellation of totals).  S and F are double-buffered per
// chain: a step writes the proposal's S' and F' into the chain's spare
// buffer and an acceptance flips the chain's buffer index.  A step is
//   move_delta_kernel  pair terms of the moved atom (old and new position);
//                      the last CTA of each chain forms dS, S' and F'
//   move_gram_kernel   dF.v and dF^T M (F + F') for 8 chains per CTA; the
//                      last CTA of each 8 chains sums them, evaluates the
//                      potential and applies the Metropolis test
// with no host round trip, so any number of steps can be enqueued at once or
// captured in a CUDA graph.  Proposals come from a counter-based generator
// (Philox4x32-10) keyed by the caller's seed and counted per chain, so a run
// is reproducible and independent of how steps are batched into calls.
// FP64 is used only for the persistent sums: on this part an FP64 FMA has a
// latency of about 64 cycles (FP32: under 5), a division about 430 and a
// square root about 670, and the FP64 pipe is shared by all warps of an SM,
// so nothing on a step's critical path computes in FP64.
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
//   log u = logf(u), u the float in (0, 1) of r1.y (FP32: a Metropolis test
//           needs no finer u, and FP64 log costs about a microsecond here)
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
  p.logu = (double)logf(unit_float(r1.y));
  return p;
}

// Chain state inside the caller's state buffer (doubles):
//   v [K], goo, 1/goo, S [2][B][K], (u, q, ee, 0) [B], F [2][B][K] as
//   floats, cur [B] as int32 (which of the two S / F buffers is the chain's
//   state).
struct MhState {
  double *v, *goo, *S, *uq;
  float *F;
  int *cur;
};

__host__ __device__ inline size_t mh_state_doubles(int n_chains, int n_bins) {
  const size_t bk = (size_t)n_chains * n_bins;
  return (size_t)n_bins + 2 + 2 * bk + 4 * (size_t)n_chains + bk +
         ((size_t)n_chains + 1) / 2;
}

__host__ __device__ inline MhState mh_state(double *base, int n_chains,
                                            int n_bins) {
  const size_t bk = (size_t)n_chains * n_bins;
  MhState st;
  st.v = base;
  st.goo = base + n_bins;
  st.S = base + n_bins + 2;
  st.uq = st.S + 2 * bk;
  st.F = reinterpret_cast<float *>(st.uq + 4 * (size_t)n_chains);
  st.cur = reinterpret_cast<int *>(st.uq + 4 * (size_t)n_chains + bk);
  return st;
}

// Row of chain b in buffer `which` of a [2][B][K] array.
__device__ __forceinline__ size_t mh_row(int which, int b, int n_chains,
                                         int n_bins) {
  return ((size_t)which * n_chains + b) * n_bins;
}

// Moves with host-chosen proposals (one per chain): mode, atom index within
// the configuration, species of an inserted atom; its position in xyz; na of
// the configuration after the move (insertion and removal change it).
enum { kMoveDisplace = 0, kMoveInsert = 1, kMoveRemove = 2 };
struct HostMoves {
  const int4 *prop;    // (mode, atom, new species, 0) per chain, or NULL
  const float4 *xyz;   // new position (displace, insert)
  const double *na;    // [n_chains][n_bins] after the move, or NULL
};

// Pair terms of the moved atom.  One CTA per work item (chain, species,
// tiles [t0, t1) of that species: consecutive sorted atoms) and bin block;
// thread (chunk c, group g) accumulates bins [kbase, kbase + L) of
//   sum_j w(|x' - x_j|) - w(|x - x_j|)
// over the atoms j = g, g + n_groups, ... of the item, with the packed
// even/odd recurrence of pair_math.cuh for both sinusoids.  The groups are
// reduced through shared memory and the CTA writes one partial row, already
// weighted by its species' form factor (FP32: a partial is a difference of a
// few hundred terms, far below S itself).  The moved atom itself contributes
// nothing (its records are zero); with host moves an inserted atom has no
// old terms and a removed one no new terms (zero records), so the rows hold
// +new or -old.  The last CTA of a chain to finish
// (counted in done[chain], which it resets) then writes, for k >= kmin, into
// the chain's spare buffer
//   S'_k = S_k + f_sa(Q_k) sum_{items of the chain} partial[item][k]
//   F'_k = 2 nan_to_num(float(S'_k) / float(na_k)),
// and F_k + F'_k, F'_k - F_k into rows of stride kp (a multiple of 4) of
// fsum and fdif.
// Dynamic shared memory: 4 * kMoveTiles * 32 float4 records +
// L * (blockDim + 1) floats.
__global__ void __launch_bounds__(kBlock)
    move_delta_kernel(const float *__restrict__ pos,
                      const int *__restrict__ perm,
                      const int4 *__restrict__ tiles,
                      const int4 *__restrict__ mitems,
                      const int *__restrict__ mitem_begin,
                      const int *__restrict__ offsets,
                      const int *__restrict__ species,
                      const unsigned long long *__restrict__ counter,
                      uint32_t seed_lo, uint32_t seed_hi, float sigma,
                      float dq_hi, float dq_lo, int kb0, int kmin,
                      int n_chunks, int n_groups, int n_bins,
                      const float *__restrict__ ftab,
                      const double *__restrict__ na,
                      MhState st, int n_chains, int kp, HostMoves hm,
                      MoveProposal *__restrict__ prop_out,
                      float *__restrict__ partial, int *__restrict__ done,
                      float *__restrict__ fsum, float *__restrict__ fdif) {
  constexpr int L = kMoveL;
  constexpr int M = L / 2;
  constexpr int NJ = kMoveTiles * kTile;
  static_assert(2 * NJ <= kBlock, "one record per thread");
  extern __shared__ float4 smem[];
  float4 *oA = smem;
  float4 *oB = oA + NJ;
  float4 *nA = oB + NJ;
  float4 *nB = nA + NJ;
  float *red = reinterpret_cast<float *>(nB + NJ);  // [j][thread], padded
  const int rs = blockDim.x + 1;
  __shared__ float sx[6];
  __shared__ int s_atom, s_last, s_mode, s_sa;

  const int4 it = mitems[blockIdx.x];  // (chain, species, t0, t1)
  const int chain = it.x;
  const int tid = threadIdx.x;
  const int s0 = tiles[it.z].x;
  const int4 tl = tiles[it.w - 1];
  const int nj = tl.x + tl.y - s0;
  // the record atom of this thread (loaded while thread 0 forms the proposal)
  const bool has_rec = tid < 2 * nj;
  const int q_rec = tid < nj ? tid : tid - nj;
  int o_rec = -1;
  float xr = 0.f, yr = 0.f, zr = 0.f;
  if (has_rec) {
    o_rec = perm[s0 + q_rec];
    xr = pos[3 * o_rec];
    yr = pos[3 * o_rec + 1];
    zr = pos[3 * o_rec + 2];
  }
  if (tid == 0) {
    const int base = offsets[chain];
    const int n = offsets[chain + 1] - base;
    if (hm.prop) {
      const int4 h = hm.prop[chain];
      const float4 xyz = hm.xyz[chain];
      const int a = (h.x == kMoveInsert) ? -1 : base + h.y;
      s_mode = h.x;
      s_atom = a;
      s_sa = (h.x == kMoveInsert) ? h.z : species[a];
      sx[0] = a >= 0 ? pos[3 * a] : 0.f;
      sx[1] = a >= 0 ? pos[3 * a + 1] : 0.f;
      sx[2] = a >= 0 ? pos[3 * a + 2] : 0.f;
      sx[3] = xyz.x;
      sx[4] = xyz.y;
      sx[5] = xyz.z;
    } else {
      const MoveProposal p =
          make_proposal(seed_lo, seed_hi, counter[chain], chain, n, sigma);
      if (blockIdx.y == 0 && (int)blockIdx.x == mitem_begin[chain])
        prop_out[chain] = p;
      const int a = base + p.atom;  // items exist only for n >= 1
      s_mode = kMoveDisplace;
      s_atom = a;
      s_sa = species[a];
      const float x = pos[3 * a], y = pos[3 * a + 1], z = pos[3 * a + 2];
      sx[0] = x;
      sx[1] = y;
      sx[2] = z;
      sx[3] = __fadd_rn(x, p.d[0]);
      sx[4] = __fadd_rn(y, p.d[1]);
      sx[5] = __fadd_rn(z, p.d[2]);
    }
  }
  __syncthreads();
  const int a = s_atom;
  const int mode = s_mode;
  // records: thread w < nj the old position, nj <= w < 2 nj the new one
  // (2 nj <= blockDim.x: at most kMoveTiles * 32 atoms per item)
  if (has_rec) {
    const bool nw = tid >= nj;
    float4 *rA = nw ? nA : oA;
    float4 *rB = nw ? nB : oB;
    if (o_rec == a || mode == (nw ? kMoveRemove : kMoveInsert)) {
      rA[q_rec] = make_float4(0.f, 0.f, 0.f, 1.f);
      rB[q_rec] = make_float4(0.f, 0.f, 0.f, 0.f);
    } else {
      const float *xs = nw ? sx + 3 : sx;
      float dx, dy, dz;
      const PairPhase2 p =
          pair_phase2(xs[0], xs[1], xs[2], xr, yr, zr, dq_hi, dq_lo, dx, dy, dz);
      rA[q_rec] = make_float4(p.th_hi, p.th_lo, p.kappa, p.sigma2);
      rB[q_rec] = make_float4(p.ch * p.inv_r, p.sh * p.inv_r, p.inv_r, 0.f);
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
      // the difference of the two terms is formed first, so that it is
      // exactly zero when the atom does not move
#pragma unroll
      for (int m = 0; m < M; ++m) {
        if (m & 1)
          acc[m] = __fadd2_rn(acc[m], __ffma2_rn(to, sgo, __fmul2_rn(tn, sgn)));
        else
          acc[m] = __fadd2_rn(acc[m], __ffma2_rn(to, f2(-1.f), tn));
        if (m + 1 < M) {
          wn = __ffma2_rn(kmn, tn, wn);
          tn = __ffma2_rn(kpn, wn, tn);
          wo = __ffma2_rn(kmo, to, wo);
          to = __ffma2_rn(kpo, wo, to);
        }
      }
    }
  }
#pragma unroll
  for (int m = 0; m < M; ++m) {
    red[(2 * m) * rs + tid] = acc[m].x;
    red[(2 * m + 1) * rs + tid] = acc[m].y;
  }
  __syncthreads();
  const int nk = n_chunks * L;
  const int kfirst = kb0 + blockIdx.y * nk;
  float *out = partial + (size_t)blockIdx.x * n_bins;
  const float *fs = ftab + (size_t)it.y * n_bins;
  for (int i = tid; i < nk; i += blockDim.x) {
    const int k = kfirst + i;
    if (k >= n_bins) continue;
    const int cc = i / L, j = i - cc * L;
    float sum = 0.f;
    for (int gg = 0; gg < n_groups; ++gg) sum += red[j * rs + gg * n_chunks + cc];
    out[k] = fs[k] * sum;
  }

  // the last CTA of the chain forms dS and F'
  __threadfence();
  __syncthreads();
  if (tid == 0) {
    const int total = (mitem_begin[chain + 1] - mitem_begin[chain]) * gridDim.y;
    s_last = (atomicAdd(done + chain, 1) == total - 1);
  }
  __syncthreads();
  if (!s_last) return;
  if (tid == 0) done[chain] = 0;
  const int sa = s_sa;
  const int i0 = mitem_begin[chain], i1 = mitem_begin[chain + 1];
  const int cb = st.cur[chain];
  const double *Sc = st.S + mh_row(cb, chain, n_chains, n_bins);
  const float *Fc = st.F + mh_row(cb, chain, n_chains, n_bins);
  double *Sn = st.S + mh_row(1 - cb, chain, n_chains, n_bins);
  float *Fn = st.F + mh_row(1 - cb, chain, n_chains, n_bins);
  const double *nab = (hm.na ? hm.na : na) + (size_t)chain * n_bins;
  float *fs_row = fsum + (size_t)chain * kp;
  float *fd_row = fdif + (size_t)chain * kp;
  for (int k = kmin + tid; k < n_bins; k += blockDim.x) {
    float d = 0.f;
#pragma unroll 4
    for (int i = i0; i < i1; ++i) d += __ldcg(partial + (size_t)i * n_bins + k);
    const double sn = Sc[k] + (double)(ftab[sa * n_bins + k] * d);
    const float fn = fq_value(sn, nab[k]);
    const float fc = Fc[k];
    Sn[k] = sn;
    Fn[k] = fn;
    fs_row[k] = fc + fn;
    fd_row[k] = fn - fc;
  }
}


constexpr int kGramCH = 8;  // chains per CTA of move_gram_kernel
constexpr int kGramRB = 8;  // rows of M per CTA (one per warp)

// Potential of a state from its Gram scalars u = G.gobs, q = G.G and
// ee = goo - u^2 / q (|gobs - s G|^2 at the optimal scale s = u / q):
//   u / q > 0:  Rw = sqrt(ee / goo), chi^2 = ee, scale u / q;
//   otherwise the reference's rules: Rw = 1, chi^2 = goo - 2 u + q (scale 1);
//   NaN stays NaN.
// The values are formed in FP32 from the FP64 state (the same expressions at
// initialisation and in the step, so that an unchanged state keeps bitwise
// the same potential).
__device__ __forceinline__ void gram_value(double u, double q, double ee,
                                           double goo, float inv_goo,
                                           int potential, double &value,
                                           double &scale) {
  const float uf = (float)u, qf = (float)q;
  if (uf > 0.f && qf > 0.f) {
    const float ef = fmaxf((float)ee, 0.f);
    value = (potential == 0) ? (double)sqrtf(ef * inv_goo) : (double)ef;
    scale = (double)(uf / qf);
  } else if (uf != uf || qf != qf || (qf == 0.f && uf == 0.f)) {
    value = scale = __longlong_as_double(0x7ff8000000000000ll);  // NaN
  } else {
    value = (potential == 0) ? 1.0 : goo - 2.0 * u + q;
    scale = 1.0;
  }
}

// dF.v and dF^T M (F + F') for 8 chains and 8 rows of M per CTA (one row k
// per warp; each lane sums M[k][l] (F + F')_l over its columns for the 8
// chains, scales by dF_k, and one recursive-halving shuffle per warp leaves
// the 8 chain sums in lanes 0, 4, ..., 28): gpart[rb][b] = (du, dq)
// (FP32: these are small increments).
// F + F' and dF come as rows of stride kp (zero where never written).
// The last CTA of the 8 chains (counted in done[blockIdx.y], which it
// resets) sums the row blocks in a fixed order, one warp per chain, and
// forms ee' - ee from the increments (FP32; the FP64 expressions of the
// reference's rules when a scale is not positive), V' and V' - V; it
// accepts when log u < -beta (V' - V), beta = conv / kT (never for a NaN
// potential); on acceptance the atom moves, the chain's buffer index flips
// and (u, q, ee) and energy = (V', scale) are updated.  The chain's proposal
// counter advances either way; chains with fewer than two atoms never move.
// trace (optional) [n_chains][8]: atom, x', y', z', log u, V', accepted, V.
// grid (ceil((n_bins - kmin) / 8), ceil(n_chains / 8)), 256 threads,
// dynamic shared memory 2 * 8 * kp floats.
constexpr int kGramNL = 12;  // column loads in flight per lane and row

__global__ void __launch_bounds__(256)
    move_gram_kernel(const float *__restrict__ M32,
                     const float *__restrict__ fsum,
                     const float *__restrict__ fdif, int kp,
                     const int *__restrict__ offsets,
                     const MoveProposal *__restrict__ prop, MhState st,
                     int n_chains, int n_bins, int kmin, int potential,
                     double beta, float *__restrict__ gpart,
                     int *__restrict__ done, float *__restrict__ pos,
                     double *__restrict__ energy,
                     unsigned long long *__restrict__ counter,
                     long long *__restrict__ accepted,
                     double *__restrict__ trace,
                     double *__restrict__ eval_out) {
  extern __shared__ float4 sm4[];
  float *ssum = reinterpret_cast<float *>(sm4);  // [l][8]: F + F'
  float *sdif = ssum + 8 * kp;                   // [l][8]: dF
  __shared__ float red[8][kGramCH][2];
  __shared__ int s_last;
  const int nkk = n_bins - kmin;
  const int b0 = blockIdx.y * kGramCH;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row = blockIdx.x * kGramRB + warp;
  // loads of the epilogue, issued first
  const float vk = (row < nkk && lane < kGramCH) ? (float)st.v[kmin + row] : 0.f;
  const int kp4 = kp >> 2;
#pragma unroll 3
  for (int idx = threadIdx.x; idx < kGramCH * kp4; idx += blockDim.x) {
    const int c = idx & 7, j = idx >> 3;
    const int b = b0 + c;
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f), d = a;
    if (b < n_chains) {
      a = reinterpret_cast<const float4 *>(fsum + (size_t)b * kp)[j];
      d = reinterpret_cast<const float4 *>(fdif + (size_t)b * kp)[j];
    }
    const float av[4] = {a.x, a.y, a.z, a.w}, dv[4] = {d.x, d.y, d.z, d.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int k = 4 * j + i;
      if (k >= kmin && k < n_bins) {  // shared row k - kmin
        ssum[(k - kmin) * 8 + c] = av[i];
        sdif[(k - kmin) * 8 + c] = dv[i];
      }
    }
  }
  __syncthreads();
  // the chain whose sum this lane holds after the halving (lanes 4c' ...)
  const int hc = ((lane >> 4) & 1) * 4 + ((lane >> 3) & 1) * 2 + ((lane >> 2) & 1);
  float v[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  float du = 0.f;
  if (row < nkk) {
    const float *mrow = M32 + (size_t)(kmin + row) * n_bins + kmin;
    for (int base = 0; base < nkk; base += 32 * kGramNL) {
      float m[kGramNL];
#pragma unroll
      for (int i = 0; i < kGramNL; ++i) {
        const int l = base + lane + 32 * i;
        m[i] = l < nkk ? mrow[l] : 0.f;
      }
#pragma unroll
      for (int i = 0; i < kGramNL; ++i) {
        const int l = base + lane + 32 * i;
        if (l >= nkk) break;
        const float4 f0 = sm4[2 * l], f1 = sm4[2 * l + 1];
        v[0] = fmaf(m[i], f0.x, v[0]);
        v[1] = fmaf(m[i], f0.y, v[1]);
        v[2] = fmaf(m[i], f0.z, v[2]);
        v[3] = fmaf(m[i], f0.w, v[3]);
        v[4] = fmaf(m[i], f1.x, v[4]);
        v[5] = fmaf(m[i], f1.y, v[5]);
        v[6] = fmaf(m[i], f1.z, v[6]);
        v[7] = fmaf(m[i], f1.w, v[7]);
      }
    }
#pragma unroll
    for (int c = 0; c < 8; ++c) v[c] *= sdif[row * 8 + c];
    if (lane < kGramCH) du = sdif[row * 8 + lane] * vk;
  }
  // recursive halving: 8 sums over 32 lanes in 4 + 2 + 1 + 1 + 1 shuffles
  {
    const bool up = lane & 16;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float give = up ? v[i] : v[i + 4];
      const float keep = up ? v[i + 4] : v[i];
      v[i] = keep + __shfl_xor_sync(0xffffffffu, give, 16);
    }
  }
  {
    const bool up = lane & 8;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const float give = up ? v[i] : v[i + 2];
      const float keep = up ? v[i + 2] : v[i];
      v[i] = keep + __shfl_xor_sync(0xffffffffu, give, 8);
    }
  }
  {
    const bool up = lane & 4;
    const float give = up ? v[0] : v[1];
    const float keep = up ? v[1] : v[0];
    v[0] = keep + __shfl_xor_sync(0xffffffffu, give, 4);
  }
  v[0] += __shfl_xor_sync(0xffffffffu, v[0], 2);
  v[0] += __shfl_xor_sync(0xffffffffu, v[0], 1);
  if ((lane & 3) == 0) red[warp][hc][1] = v[0];
  if (lane < kGramCH) red[warp][lane][0] = du;
  __syncthreads();
  if (threadIdx.x < kGramCH * 2) {
    const int c = threadIdx.x >> 1, j = threadIdx.x & 1;
    const int b = b0 + c;
    if (b < n_chains) {
      float sum = 0.f;
      for (int w = 0; w < 8; ++w) sum += red[w][c][j];
      gpart[((size_t)blockIdx.x * n_chains + b) * 2 + j] = sum;
    }
  }

  // the last CTA of these chains: potential and Metropolis test
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0)
    s_last = (atomicAdd(done + blockIdx.y, 1) == (int)gridDim.x - 1);
  __syncthreads();
  if (!s_last) return;
  if (threadIdx.x == 0) done[blockIdx.y] = 0;
  const int b = b0 + warp;  // one warp per chain
  if (b >= n_chains) return;
  // per-chain values, loaded by lane 0 before the reduction
  int o0 = 0, o1 = 0, cb = 0;
  double u0 = 0.0, q0 = 0.0, ee0 = 0.0, e0 = 0.0, goo = 0.0;
  float inv_goo = 0.f;
  MoveProposal p;
  if (lane == 0) {
    o0 = offsets[b];
    o1 = offsets[b + 1];
    cb = st.cur[b];
    u0 = st.uq[4 * b];
    q0 = st.uq[4 * b + 1];
    ee0 = st.uq[4 * b + 2];
    e0 = energy ? energy[2 * b] : 0.0;
    goo = st.goo[0];
    inv_goo = (float)st.goo[1];
    p = prop[b];
  }
  float su = 0.f, sq = 0.f;
  for (int rb = lane; rb < (int)gridDim.x; rb += 32) {
    const float2 g = __ldcg(reinterpret_cast<const float2 *>(gpart) +
                            (size_t)rb * n_chains + b);
    su += g.x;
    sq += g.y;
  }
  for (int o = 16; o > 0; o >>= 1) {
    su += __shfl_xor_sync(0xffffffffu, su, o);
    sq += __shfl_xor_sync(0xffffffffu, sq, o);
  }
  if (lane != 0) return;
  double *tr = trace ? trace + (size_t)b * 8 : nullptr;
  if (eval_out) {
    // evaluation only (host-chosen moves): the proposal's potential and Gram
    // scalars, no state change
    double *ev = eval_out + (size_t)b * 8;
    const double nan = __longlong_as_double(0x7ff8000000000000ll);
    double value = nan, scale = nan, u1 = nan, q1 = nan, ee1 = nan;
    if (o1 - o0 >= 1) {
      u1 = u0 + (double)su;
      q1 = q0 + (double)sq;
      const float uf = (float)u0, qf = (float)q0;
      const float u1f = uf + su, q1f = qf + sq;
      if (uf > 0.f && qf > 0.f && u1f > 0.f && q1f > 0.f) {
        const float dee = -(fmaf(2.f * uf, su, su * su) * qf - uf * uf * sq) /
                          (qf * q1f);
        ee1 = ee0 + (double)dee;
      } else {
        ee1 = goo - u1 * u1 / q1;
      }
      gram_value(u1, q1, ee1, goo, inv_goo, potential, value, scale);
    }
    ev[0] = value;
    ev[1] = scale;
    ev[2] = u1;
    ev[3] = q1;
    ev[4] = ee1;
    ev[5] = e0;
    return;
  }
  if (o1 - o0 < 2) {
    counter[b] += 1ull;
    if (tr)
      for (int i = 0; i < 8; ++i) tr[i] = 0.0;
    return;
  }
  const int at = o0 + p.atom;
  float xn[3];
  for (int i = 0; i < 3; ++i) xn[i] = __fadd_rn(pos[3 * at + i], p.d[i]);
  const float uf = (float)u0, qf = (float)q0;
  const float u1f = uf + su, q1f = qf + sq;
  double value, scale, u1, q1, ee1;
  float dv;  // V' - V for the test
  if (uf > 0.f && qf > 0.f && u1f > 0.f && q1f > 0.f) {
    // increments only: ee' - ee = -[(2 u du + du^2) q - u^2 dq] / (q q')
    const float dee = -(fmaf(2.f * uf, su, su * su) * qf - uf * uf * sq) /
                      (qf * q1f);
    const float ef = fmaxf((float)ee0 + dee, 0.f);
    const float ve = (float)e0;
    if (potential == 0) {
      const float v1 = sqrtf(ef * inv_goo);
      const float den = v1 + ve;
      dv = den > 0.f ? dee * inv_goo / den : 0.f;
      value = (double)v1;
    } else {
      dv = dee;
      value = (double)ef;
    }
    scale = (double)(u1f / q1f);
    u1 = u0 + (double)su;
    q1 = q0 + (double)sq;
    ee1 = ee0 + (double)dee;
  } else {
    // a non-positive or undefined scale on either side: the reference's
    // rules in FP64 (rare)
    u1 = u0 + (double)su;
    q1 = q0 + (double)sq;
    ee1 = goo - u1 * u1 / q1;
    gram_value(u1, q1, ee1, goo, inv_goo, potential, value, scale);
    dv = (float)(value - e0);
  }
  const bool acc = (float)p.logu < -(float)beta * dv;
  if (acc) {
    for (int i = 0; i < 3; ++i) pos[3 * at + i] = xn[i];
    st.cur[b] = 1 - cb;
    st.uq[4 * b] = u1;
    st.uq[4 * b + 1] = q1;
    st.uq[4 * b + 2] = ee1;
    energy[2 * b] = value;
    energy[2 * b + 1] = scale;
    accepted[b] += 1;
  }
  if (tr) {
    tr[0] = (double)p.atom;
    tr[1] = xn[0];
    tr[2] = xn[1];
    tr[3] = xn[2];
    tr[4] = p.logu;
    tr[5] = value;
    tr[6] = acc ? 1.0 : 0.0;
    tr[7] = e0;
  }
  counter[b] += 1ull;
}

// Host decision on host-chosen moves: for chains with accept[b] != 0 the
// proposal evaluated by move_gram_kernel (eval[b] = V', scale, u', q', ee')
// becomes the state: the buffer index flips, (u, q, ee) and energy are stored.
__global__ void mh_commit_kernel(const int *__restrict__ accept,
                                 const double *__restrict__ eval, MhState st,
                                 double *__restrict__ energy, int n_chains) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n_chains || !accept[b]) return;
  const double *ev = eval + (size_t)b * 8;
  st.cur[b] = 1 - st.cur[b];
  st.uq[4 * b] = ev[2];
  st.uq[4 * b + 1] = ev[3];
  st.uq[4 * b + 2] = ev[4];
  energy[2 * b] = ev[0];
  energy[2 * b + 1] = ev[1];
}

// ---------------------------------------------------------- state set-up
// M64[k][l] = sum_i T[k][i] T[l][i] in FP64 (exact products of the float T),
// 32 x 32 tiles, 32 x 8 threads with 4 rows each; M32 = float(M64).
__global__ void gram_matrix_kernel(const float *__restrict__ T, int n_bins,
                                   int n_r, double *__restrict__ M64,
                                   float *__restrict__ M32) {
  __shared__ float ta[32][33], tb[32][33];
  const int k0 = blockIdx.y * 32, l0 = blockIdx.x * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int i0 = 0; i0 < n_r; i0 += 32) {
    for (int r = ty; r < 32; r += 8) {
      const int i = i0 + tx;
      ta[r][tx] = (k0 + r < n_bins && i < n_r) ? T[(size_t)(k0 + r) * n_r + i] : 0.f;
      tb[r][tx] = (l0 + r < n_bins && i < n_r) ? T[(size_t)(l0 + r) * n_r + i] : 0.f;
    }
    __syncthreads();
    for (int ii = 0; ii < 32; ++ii) {
      const double bv = (double)tb[tx][ii];
#pragma unroll
      for (int m = 0; m < 4; ++m)
        acc[m] = fma((double)ta[ty + 8 * m][ii], bv, acc[m]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    const int k = k0 + ty + 8 * m, l = l0 + tx;
    if (k < n_bins && l < n_bins) {
      M64[(size_t)k * n_bins + l] = acc[m];
      M32[(size_t)k * n_bins + l] = (float)acc[m];
    }
  }
}

// v[k] = sum_i T[k][i] gobs[i] (block k < n_bins) and goo = gobs.gobs
// (block n_bins), FP64.
__global__ void mh_gobs_kernel(const float *__restrict__ T,
                               const double *__restrict__ gobs, int n_bins,
                               int n_r, MhState st) {
  __shared__ double scratch[32];
  const int k = blockIdx.x;
  double a[1] = {0.0};
  if (k < n_bins) {
    for (int i = threadIdx.x; i < n_r; i += blockDim.x)
      a[0] += (double)T[(size_t)k * n_r + i] * gobs[i];
  } else {
    for (int i = threadIdx.x; i < n_r; i += blockDim.x) a[0] += gobs[i] * gobs[i];
  }
  block_sum<1>(a, scratch);
  if (threadIdx.x == 0) {
    if (k < n_bins)
      st.v[k] = a[0];
    else {
      st.goo[0] = a[0];
      st.goo[1] = 1.0 / a[0];
    }
  }
}

// Per chain (one CTA): u = v.F, q = F^T M64 F, ee = goo - u^2 / q (FP64) of
// buffer 0, cur = 0, and the potential of the state into energy.
__global__ void mh_init_kernel(const double *__restrict__ M64, MhState st,
                               int n_chains, int n_bins, int potential,
                               double *__restrict__ energy) {
  __shared__ double scratch[32 * 2];
  const int b = blockIdx.x;
  const float *F = st.F + mh_row(0, b, n_chains, n_bins);
  double a2[2] = {0.0, 0.0};
  for (int k = threadIdx.x; k < n_bins; k += blockDim.x) {
    const double *mr = M64 + (size_t)k * n_bins;
    double yk = 0.0;
    for (int l = 0; l < n_bins; ++l) yk = fma(mr[l], (double)F[l], yk);
    a2[0] += st.v[k] * (double)F[k];
    a2[1] += yk * (double)F[k];
  }
  block_sum<2>(a2, scratch);
  if (threadIdx.x == 0) {
    const double u = a2[0], q = a2[1], goo = st.goo[0];
    const double ee = goo - u * u / q;
    st.cur[b] = 0;
    st.uq[4 * b] = u;
    st.uq[4 * b + 1] = q;
    st.uq[4 * b + 2] = ee;
    st.uq[4 * b + 3] = 0.0;
    double value, scale;
    gram_value(u, q, ee, goo, (float)st.goo[1], potential, value, scale);
    energy[2 * b] = value;
    energy[2 * b + 1] = scale;
  }
}

}  // namespace pyiid
