// Host build of pyiid_gb300/csrc/pair_math.cuh for tests/test_pair_math_cpu.py.
//
// The header's arithmetic uses only correctly rounded intrinsics (__fadd_rn,
// __fmul_rn, __fmaf_rn, __fsqrt_rn, __frcp_rn, ...), whose results are fixed
// by IEEE 754, so compiled here with the matching host operations (and
// -ffp-contract=off) it gives the device's values bit for bit.  The one
// exception is the hardware sin/cos of the seeds (__sincosf), replaced by the
// host's sin/cos: the figures for the seeds below measure the phase
// reduction, not the hardware sin/cos.
//
// Prints one JSON object of maximum errors against FP64 truth over random
// pairs (cube edges up to 200 A, the grid steps of the tests and the bench)
// and a dense grid of the half-angle sin/cos argument.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <random>

static inline float __fadd_rn(float a, float b) { return a + b; }
static inline float __fsub_rn(float a, float b) { return a - b; }
static inline float __fmul_rn(float a, float b) { return a * b; }
static inline float __fdiv_rn(float a, float b) { return a / b; }
static inline float __fmaf_rn(float a, float b, float c) {
  return std::fma(a, b, c);
}
static inline float __frcp_rn(float a) { return 1.0f / a; }
static inline float __fsqrt_rn(float a) { return std::sqrt(a); }
static inline void host_sincosf(float x, float *s, float *c) {
  *s = (float)std::sin((double)x);
  *c = (float)std::cos((double)x);
}
#define __sincosf host_sincosf

#include "pair_math.cuh"

using pyiid::PairPhase2;

int main(int argc, char **argv) {
  const int n_pairs = argc > 1 ? std::atoi(argv[1]) : 200000;
  const unsigned seed = argc > 2 ? (unsigned)std::atoi(argv[2]) : 1u;
  std::mt19937_64 rng(seed);
  std::uniform_real_distribution<double> u01(0.0, 1.0);
  const double steps[] = {0.02, 0.05, 0.1, 0.13, 0.0756865};
  const double edges[] = {4.0, 20.0, 80.0, 200.0};

  double e_r = 0, e_th = 0, e_sth = 0, e_cth = 0, e_norm = 0, e_s2 = 0,
         e_c2 = 0, e_seed = 0, e_seed_odd = 0, e_theta2 = 0, e_kappa = 0;
  double th_max = 0;
  for (int i = 0; i < n_pairs; ++i) {
    const double dq = steps[i % 5];
    const double edge = edges[(i / 5) % 4];
    float a[3], b[3];
    for (int c = 0; c < 3; ++c) {
      a[c] = (float)((u01(rng) - 0.5) * edge);
      b[c] = (float)((u01(rng) - 0.5) * edge);
    }
    const float dq_hi = (float)dq;
    const float dq_lo = (float)(dq - (double)dq_hi);
    float dx, dy, dz;
    const PairPhase2 p = pyiid::pair_phase2(a[0], a[1], a[2], b[0], b[1],
                                            b[2], dq_hi, dq_lo, dx, dy, dz);
    // FP64 truth from the same float positions (differences exact in double)
    const double tx = (double)a[0] - b[0], ty = (double)a[1] - b[1],
                 tz = (double)a[2] - b[2];
    const double r = std::sqrt(tx * tx + ty * ty + tz * tz);
    if (r < 1e-3) continue;
    const double th = ((double)dq_hi + (double)dq_lo) * r;
    th_max = std::fmax(th_max, th);
    e_r = std::fmax(e_r, std::fabs((double)p.r - r) / r);
    const double thp = (double)p.th_hi + (double)p.th_lo;
    e_th = std::fmax(e_th, std::fabs(thp - th) / th);
    e_sth = std::fmax(e_sth, std::fabs((double)p.sth - std::sin(th)));
    e_cth = std::fmax(e_cth, std::fabs((double)p.cth - std::cos(th)));
    const double sh = p.sh, ch = p.ch;
    e_norm = std::fmax(e_norm, std::fabs(sh * sh + ch * ch - 1.0));
    // (sigma2, theta2) reproduce the step 2 theta: sigma2 sin theta2 =
    // sin 2theta and sigma2 cos theta2 = cos 2theta, theta2 in [-pi/2, pi/2]
    const double s2 = 2.0 * sh * ch, c2 = ch * ch - sh * sh;
    e_s2 = std::fmax(e_s2, std::fabs(p.sigma2 * s2 - std::sin(2.0 * th)));
    e_c2 = std::fmax(e_c2, std::fabs(p.sigma2 * c2 - std::cos(2.0 * th)));
    const double theta2 = 2.0 * std::atan2(sh, ch);
    e_theta2 = std::fmax(e_theta2, std::fabs(theta2) - M_PI / 2);
    e_kappa = std::fmax(e_kappa, std::fabs((double)p.kappa - 2.0 * sh));
    // seeds at the start of every 24-bin chunk up to bin 1500
    for (int k0 = 0; k0 < 1500; k0 += 24 * 7) {
      float2 s, c;
      pyiid::seed_sincos2r((float)k0, p.th_hi, p.th_lo, p.sth, p.cth, s, c);
      const double ph0 = (double)k0 * thp, ph1 = (double)(k0 + 1) * thp;
      e_seed = std::fmax(e_seed, std::fmax(std::fabs(s.x - std::sin(ph0)),
                                           std::fabs(c.x - std::cos(ph0))));
      e_seed_odd = std::fmax(e_seed_odd,
                             std::fmax(std::fabs(s.y - std::sin(ph1)),
                                       std::fabs(c.y - std::cos(ph1))));
    }
  }
  // the half-angle series on a dense grid of [-pi/4, pi/4]
  double e_ts = 0, e_tc = 0;
  const int n_grid = 1 << 22;
  for (int i = 0; i <= n_grid; ++i) {
    const float x = (float)(-M_PI / 4 + (M_PI / 2) * i / n_grid);
    float s, c;
    pyiid::sincos_quarter_turn(x, s, c);
    e_ts = std::fmax(e_ts, std::fabs((double)s - std::sin((double)x)));
    e_tc = std::fmax(e_tc, std::fabs((double)c - std::cos((double)x)));
  }
  std::printf(
      "{\"pairs\": %d, \"theta_max\": %.6g, \"r_rel\": %.3e, "
      "\"theta_rel\": %.3e, \"sin_theta_abs\": %.3e, \"cos_theta_abs\": %.3e, "
      "\"half_angle_norm\": %.3e, \"sin_2theta_abs\": %.3e, "
      "\"cos_2theta_abs\": %.3e, \"theta2_over_half_pi\": %.3e, "
      "\"kappa_abs\": %.3e, \"seed_abs\": %.3e, \"seed_odd_abs\": %.3e, "
      "\"taylor_sin_abs\": %.3e, \"taylor_cos_abs\": %.3e}\n",
      n_pairs, th_max, e_r, e_th, e_sth, e_cth, e_norm, e_s2, e_c2, e_theta2,
      e_kappa, e_seed, e_seed_odd, e_ts, e_tc);
  return 0;
}
