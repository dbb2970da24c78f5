// pair_math.cuh -- per-pair phase arithmetic shared by the Debye kernels.
//
// Every Debye term needs sin(Q_k r) (and for gradients cos(Q_k r)) on a
// uniform grid Q_k = k*dq.  Forming the FP32 argument k*dq*r directly loses
// up to half an ulp of a number that reaches several thousand radians
// (1e-4 rad at Q*r = 2500), so the kernels never do that.  Instead, per pair:
//
//   1. r and theta = dq*r are formed as unevaluated float pairs (hi + lo)
//      with error-free transformations (TwoSum, FMA-based TwoProd), from the
//      FP32 positions the reference also uses.
//   2. theta is folded to theta_e = theta - m*pi in [-pi/2, pi/2] (Cody-Waite
//      with a three-float split of pi), sigma = (-1)^m, so that
//        sin(k theta) = sigma^k sin(k theta_e),  cos(k theta) = sigma^k cos(k theta_e).
//   3. sin(k theta_e) is generated bin by bin with Reinsch's modified
//      recurrence of the Chebyshev three-term recurrence
//        v_{k+1} = v_k + lambda t_k,  t_{k+1} = t_k + v_{k+1},
//        lambda  = -4 sin^2(theta_e/2),  v_k = t_k - t_{k-1},
//      which needs one FMA and one add per bin and, unlike the plain
//      t_{k+1} = 2cos(theta) t_k - t_{k-1}, does not amplify rounding errors
//      by 1/sin(theta) for small theta (Reinsch's modification; see e.g.
//      Oliver, "An error analysis of the modified Clenshaw method", 1977).
//      cos(k theta_e) = (v_k + v_{k+1}) / (2 sin theta_e).
//   4. The recurrence is re-seeded every L bins from sin/cos of the reduced
//      seed phase k0*theta_e (again a float pair, reduced modulo 2*pi by a
//      three-float split of 2*pi), so rounding drift is bounded by L steps.
//
// The split constants below are pi and 2*pi rounded to float, then the float
// roundings of the remainders, computed from a 60-digit value of pi.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace pyiid {

constexpr float kPiA = 3.1415927410125732f;           // 0x1.921fb6p+1
constexpr float kPiB = -8.742277657347586e-08f;       // -0x1.777a5cp-24
constexpr float kPiC = -3.4302490200117637e-15f;      // -0x1.ee59dap-49
constexpr float kTwoPiA = 6.2831854820251465f;        // 0x1.921fb6p+2
constexpr float kTwoPiB = -1.7484555314695172e-07f;   // -0x1.777a5cp-23
constexpr float kTwoPiC = -6.8604980400235275e-15f;   // -0x1.ee59dap-48
constexpr float kInvPi = 0.31830987334251404f;        // 0x1.45f306p-2
constexpr float kInvTwoPi = 0.15915493667125702f;     // 0x1.45f306p-3

// --- error-free transformations (explicit rounding intrinsics so that the
//     compiler never contracts or reassociates them) -------------------------
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void fast_two_sum(float a, float b, float &s,
                                             float &e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

__device__ __forceinline__ void two_prod(float a, float b, float &p, float &e) {
  p = __fmul_rn(a, b);
  e = __fmaf_rn(a, b, -p);
}

// Per-pair phase data.  theta_e = th_hi + th_lo in [-pi/2, pi/2].
struct PairPhase {
  float th_hi, th_lo;  // folded phase step dq*r - m*pi
  float sigma;         // (-1)^m
  float lam;           // -4 sin^2(theta_e/2)
  float sin_th;        // sin(theta_e)
  float r;             // |x_a - x_b| (FP32)
  float inv_r;         // 1 / r
};

// Builds the phase data of the pair (a, b) for the grid step dq = dq_hi + dq_lo.
// d = a - b is returned in (dx, dy, dz).  For a == b (r = 0) the returned
// inv_r is +inf and the callers' products turn into NaN exactly where the
// reference's sin(0)/0 does.
__device__ __forceinline__ PairPhase pair_phase(float ax, float ay, float az,
                                                float bx, float by, float bz,
                                                float dq_hi, float dq_lo,
                                                float &dx, float &dy,
                                                float &dz) {
  PairPhase p;
  float xl, yl, zl;
  two_sum(ax, -bx, dx, xl);
  two_sum(ay, -by, dy, yl);
  two_sum(az, -bz, dz, zl);
  // r^2 = sum (d_hi + d_lo)^2  ~= sum d_hi^2 + 2 d_hi d_lo  (d_lo^2 < 2^-48 rel.)
  float s0, e0, s1, e1, s2, e2;
  two_prod(dx, dx, s0, e0);
  two_prod(dy, dy, s1, e1);
  two_prod(dz, dz, s2, e2);
  float h, l, h2, l2;
  two_sum(s0, s1, h, l);
  two_sum(h, s2, h2, l2);
  float lo = l + l2 + e0 + e1 + e2 + 2.0f * (dx * xl + dy * yl + dz * zl);
  float r2h, r2l;
  fast_two_sum(h2, lo, r2h, r2l);
  float rh = __fsqrt_rn(r2h);
  float res = __fmaf_rn(-rh, rh, r2h);  // exact residual r2h - rh^2
  float rl = __fmul_rn(__fadd_rn(res, r2l), __fdiv_rn(0.5f, rh));
  // theta = dq * r as a float pair
  float th, tl;
  two_prod(dq_hi, rh, th, tl);
  tl = __fadd_rn(tl, __fmaf_rn(dq_hi, rl, __fmul_rn(dq_lo, rh)));
  fast_two_sum(th, tl, th, tl);
  // fold: theta_e = theta - m*pi; the first product-difference is exact
  float m = rintf(__fmul_rn(th, kInvPi));
  float x = __fmaf_rn(-m, kPiA, th);
  float y = __fmaf_rn(-m, kPiC, __fmaf_rn(-m, kPiB, tl));
  two_sum(x, y, p.th_hi, p.th_lo);
  int mi = (int)m;
  p.sigma = (mi & 1) ? -1.0f : 1.0f;
  // accurate half-angle sin/cos (full-precision sincosf), then the lo term
  float hs, hc;
  sincosf(0.5f * p.th_hi, &hs, &hc);
  float hl = 0.5f * p.th_lo;
  float hs2 = __fmaf_rn(hc, hl, hs);
  float hc2 = __fmaf_rn(-hs, hl, hc);
  p.lam = -4.0f * hs2 * hs2;
  p.sin_th = 2.0f * hs2 * hc2;
  p.r = rh;
  p.inv_r = __frcp_rn(rh);
  return p;
}

// sin and cos of k0 * theta_e (k0 an exact small integer in float) with the
// phase formed as a float pair and reduced modulo 2*pi.  The first
// product-difference of the reduction is exact; the residual phase error is a
// few 1e-7 rad, dominated by the hardware sin/cos of the reduced argument.
__device__ __forceinline__ void seed_sincos(float k0, float th_hi, float th_lo,
                                            float &s, float &c) {
  float ph = __fmul_rn(k0, th_hi);
  float pl = __fmaf_rn(k0, th_lo, __fmaf_rn(k0, th_hi, -ph));
  float n = rintf(__fmul_rn(ph, kInvTwoPi));
  float x = __fmaf_rn(-n, kTwoPiA, ph);
  x = __fmaf_rn(-n, kTwoPiB, x);
  x = __fadd_rn(x, __fmaf_rn(-n, kTwoPiC, pl));
  __sincosf(x, &s, &c);
}

// ---------------------------------------------------------------------------
// Packed even/odd formulation (FP32x2 instructions of sm_100+).
//
// The bins k = k0 + 2m + e (e = 0, 1) of one pair are two interleaved
// sinusoids in m with step 2*theta.  Folding 2*theta = theta2 + M*pi with
// theta2 in [-pi/2, pi/2] and sigma2 = (-1)^M gives
//   sin(k theta) = sigma2^m sin(phi_e + m theta2),  phi_e = (k0 + e) theta,
//   cos(k theta) = sigma2^m cos(phi_e + m theta2),
// and both slots advance with one packed instruction pair of the Minsky
// ("magic circle") recurrence with kappa = 2 sin(theta2/2):
//   w_{m+1} = w_m - kappa t_m,   t_{m+1} = t_m + kappa w_{m+1},
//   t_m = sin(phi + m theta2),   w_m = cos(phi + (m - 1/2) theta2).
// Its matrix has determinant 1 (rounding does not grow the amplitude) and it
// yields the cosine without any 1/sin(theta) factor:
//   cos(phi + m theta2) = (w_m + w_{m+1}) / (2 cos(theta2/2)).
struct PairPhase2 {
  float th_hi, th_lo;   // theta = dq * r (unfolded), seeds use it
  float sigma2;         // (-1)^M
  float kappa;          // 2 sin(theta2 / 2)
  float sh, ch;         // sin, cos of theta2 / 2
  float sth, cth;       // sin, cos of theta (a quarter-turn rotation of sh, ch)
  float r, inv_r;
};

// sin and cos of x for |x| <= pi/4 by their Taylor series about 0 through
// x^9 and x^10 (coefficients 1/n!): the first omitted terms are below 2e-9
// there, under float rounding; Horner evaluation adds about one rounding.
__device__ __forceinline__ void sincos_quarter_turn(float x, float &s,
                                                    float &c) {
  const float x2 = x * x;
  s = fmaf(x * x2,
           fmaf(x2, fmaf(x2, fmaf(x2, 2.7557319e-6f, -1.9841270e-4f),
                         8.3333333e-3f),
                -1.6666667e-1f),
           x);
  c = fmaf(x2,
           fmaf(x2,
                fmaf(x2, fmaf(x2, fmaf(x2, -2.7557319e-7f, 2.4801587e-5f),
                              -1.3888889e-3f),
                     4.1666667e-2f),
                -0.5f),
           1.0f);
}

__device__ __forceinline__ PairPhase2 pair_phase2(float ax, float ay, float az,
                                                  float bx, float by, float bz,
                                                  float dq_hi, float dq_lo,
                                                  float &dx, float &dy,
                                                  float &dz) {
  PairPhase2 p;
  float xl, yl, zl;
  two_sum(ax, -bx, dx, xl);
  two_sum(ay, -by, dy, yl);
  two_sum(az, -bz, dz, zl);
  float s0, e0, s1, e1, s2, e2;
  two_prod(dx, dx, s0, e0);
  two_prod(dy, dy, s1, e1);
  two_prod(dz, dz, s2, e2);
  float h, l, h2, l2;
  two_sum(s0, s1, h, l);
  two_sum(h, s2, h2, l2);
  float lo = l + l2 + e0 + e1 + e2 + 2.0f * (dx * xl + dy * yl + dz * zl);
  float r2h, r2l;
  fast_two_sum(h2, lo, r2h, r2l);
  float rh = __fsqrt_rn(r2h);
  float res = __fmaf_rn(-rh, rh, r2h);
  const float inv_r = __frcp_rn(rh);
  float rl = __fmul_rn(__fadd_rn(res, r2l), 0.5f * inv_r);
  float th, tl;
  two_prod(dq_hi, rh, th, tl);
  tl = __fadd_rn(tl, __fmaf_rn(dq_hi, rl, __fmul_rn(dq_lo, rh)));
  fast_two_sum(th, tl, th, tl);
  p.th_hi = th;
  p.th_lo = tl;
  // theta2 = 2 theta - M pi (doubling is exact)
  const float t2h = 2.0f * th, t2l = 2.0f * tl;
  float m = rintf(__fmul_rn(t2h, kInvPi));
  float x = __fmaf_rn(-m, kPiA, t2h);
  float y = __fmaf_rn(-m, kPiC, __fmaf_rn(-m, kPiB, t2l));
  float q_hi, q_lo;
  two_sum(x, y, q_hi, q_lo);
  int mi = (int)m;
  p.sigma2 = (mi & 1) ? -1.0f : 1.0f;
  float hs, hc;  // |q_hi| <= pi/2
  sincos_quarter_turn(0.5f * q_hi, hs, hc);
  const float hl = 0.5f * q_lo;
  p.sh = __fmaf_rn(hc, hl, hs);
  p.ch = __fmaf_rn(-hs, hl, hc);
  p.kappa = 2.0f * p.sh;
  // theta = theta2 / 2 + M pi / 2: rotate (sh, ch) by M quarter turns
  switch (mi & 3) {
    case 0: p.sth = p.sh;  p.cth = p.ch;  break;
    case 1: p.sth = p.ch;  p.cth = -p.sh; break;
    case 2: p.sth = -p.sh; p.cth = -p.ch; break;
    default: p.sth = -p.ch; p.cth = p.sh; break;
  }
  p.r = rh;
  p.inv_r = inv_r;
  return p;
}

// Seeds of both slots: (sin, cos) of k0*theta and (k0+1)*theta, each phase a
// float pair reduced modulo 2*pi as in seed_sincos.
__device__ __forceinline__ void seed_sincos2(float k0, float th_hi,
                                             float th_lo, float2 &s,
                                             float2 &c) {
  seed_sincos(k0, th_hi, th_lo, s.x, c.x);
  seed_sincos(k0 + 1.0f, th_hi, th_lo, s.y, c.y);
}

// Seeds of both slots from one reduced phase: (sin, cos) of k0*theta as in
// seed_sincos, then those of (k0+1)*theta by the angle-addition rotation with
// the pair's (sin theta, cos theta).  One reduction and one hardware sin/cos
// instead of two; the rotation adds about two roundings.
__device__ __forceinline__ void seed_sincos2r(float k0, float th_hi,
                                              float th_lo, float sth,
                                              float cth, float2 &s,
                                              float2 &c) {
  seed_sincos(k0, th_hi, th_lo, s.x, c.x);
  s.y = __fmaf_rn(c.x, sth, __fmul_rn(s.x, cth));
  c.y = __fmaf_rn(-s.x, sth, __fmul_rn(c.x, cth));
}

__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }

}  // namespace pyiid
