// transform_kernels.cuh -- F(Q) -> G(r), potentials and the adjoint weights.
//
// The reference's F -> G transform (zero pad, odd extension, inverse FFT,
// linear interpolation onto the r grid) is a fixed linear map
//   G(r_i) = sum_k F_k T[k][i]
// (see the host builder of T for the derivation): get_pdf_at_qmin,
// fft_fq_to_gr and fft_gr_to_fq of pyiid/experiments/elasticscatter/
// kernels/master_kernel.py:39-203.  T is stored [n_bins][n_r]
// in FP32, so G for a batch of configurations is a skinny GEMM streaming T
// from HBM/L2 once per CTA column block.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace pyiid {

// gr[b][i] = sum_k fq[b][k] * T[k][i]  (FP32 products, FP32 blocks of 32 bins
// summed in FP64).  grid (ceil(n_r/256), n_configs)
__global__ void pdf_kernel(const float *__restrict__ fq,
                           const float *__restrict__ T, int n_bins, int n_r,
                           int kmin, double *__restrict__ gr) {
  extern __shared__ float sf[];
  const int b = blockIdx.y;
  for (int k = threadIdx.x; k < n_bins; k += blockDim.x)
    sf[k] = (k >= kmin) ? fq[(size_t)b * n_bins + k] : 0.f;
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_r) return;
  double acc = 0.0;
  for (int k0 = kmin; k0 < n_bins; k0 += 32) {
    float part = 0.f;
    const int k1 = min(k0 + 32, n_bins);
    for (int k = k0; k < k1; ++k) part = fmaf(sf[k], T[(size_t)k * n_r + i], part);
    acc += (double)part;
  }
  gr[(size_t)b * n_r + i] = acc;
}

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double *scratch) {
  // scratch: [32][NV]
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < NV; ++i) v[i] = warp_sum(v[i]);
  if (lane == 0)
#pragma unroll
    for (int i = 0; i < NV; ++i) scratch[wid * NV + i] = v[i];
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    double s = 0.0;
    for (int w = 0; w < nw; ++w) s += scratch[w * NV + i];
    v[i] = s;
  }
  __syncthreads();
}

// Potential per configuration (one CTA each), get_rw / get_chi_sq / get_scale
// of kernels/master_kernel.py:206-266, 388-389:
//   a = (gc.go)/(gc.gc); Rw: a <= 0 -> (1, 1), else sqrt(|go - a gc|^2/|go|^2)
//   chi^2: s = a if a > 0 else 1, value = |go - s gc|^2
// Optionally the adjoint vector c = d(value)/d(gcalc) exactly as the
// reference's get_grad_rw / get_grad_chi_sq contract it (the derivative of
// the scale uses the raw a even when the value used scale 1):
//   c_i = pre [s E_i + (gc.E) (go_i - 2 a gc_i)/(gc.gc)],  E = go - s gc,
//   pre = -Rw/|E|^2 (Rw) or -2 (chi^2).
struct PotentialValue {
  double value, scale;  // potential and the scale it used
  double a, gcc, ee, gce;
};

// The potential of one configuration, computed by the whole CTA (every
// thread returns the same values).  scratch: 32 * 4 doubles of shared memory.
// weight (Rw only, may be null): per-point weights of get_rw
// (master_kernel.py:226-235): Rw = sqrt(sum w (go - a gc)^2 / sum w go^2)
// with the unweighted scale a; ee and gce (used by the gradients, which the
// reference never weights) stay unweighted.
__device__ __forceinline__ PotentialValue potential_value(
    const double *__restrict__ gobs, const double *__restrict__ gc, int n_r,
    int potential, double *scratch,
    const double *__restrict__ weight = nullptr) {
  double v3[4] = {0.0, 0.0, 0.0, 0.0};
  for (int i = threadIdx.x; i < n_r; i += blockDim.x) {
    const double c = gc[i], o = gobs[i];
    v3[0] += c * o;
    v3[1] += c * c;
    v3[2] += o * o;
    if (weight) v3[3] += weight[i] * o * o;
  }
  block_sum<4>(v3, scratch);
  const double gco = v3[0], gcc = v3[1];
  const double goo = weight ? v3[3] : v3[2];
  const double a = gco / gcc;
  // the reference replaces a non-positive scale by 1; a NaN scale stays NaN
  const double s = (a <= 0.0) ? 1.0 : a;
  double v2[3] = {0.0, 0.0, 0.0};
  for (int i = threadIdx.x; i < n_r; i += blockDim.x) {
    const double e = gobs[i] - s * gc[i];
    v2[0] += e * e;
    v2[1] += gc[i] * e;
    if (weight) v2[2] += weight[i] * e * e;
  }
  block_sum<3>(v2, scratch);
  PotentialValue r;
  r.ee = v2[0];
  r.gce = v2[1];
  r.a = a;
  r.gcc = gcc;
  r.scale = s;
  const double top = weight ? v2[2] : v2[0];
  if (potential == 0)
    r.value = (a <= 0.0) ? 1.0 : sqrt(top / goo);
  else
    r.value = r.ee;
  return r;
}

__global__ void potential_kernel(const double *__restrict__ gobs,
                                 const double *__restrict__ gcalc, int n_r,
                                 int potential, double *__restrict__ out,
                                 float *__restrict__ cvec,
                                 const double *__restrict__ weight = nullptr) {
  __shared__ double scratch[32 * 4];
  const int b = blockIdx.x;
  const double *gc = gcalc + (size_t)b * n_r;
  const PotentialValue pv =
      potential_value(gobs, gc, n_r, potential, scratch, weight);
  const double value = pv.value, s = pv.scale, a = pv.a, gcc = pv.gcc;
  const double ee = pv.ee, gce = pv.gce;
  const double pre = (potential == 0) ? -value / ee : -2.0;
  if (threadIdx.x == 0) {
    out[2 * b] = value;
    out[2 * b + 1] = s;
  }
  if (cvec) {
    for (int i = threadIdx.x; i < n_r; i += blockDim.x) {
      const double e = gobs[i] - s * gc[i];
      const double ci = pre * (s * e + gce * (gobs[i] - 2.0 * a * gc[i]) / gcc);
      cvec[(size_t)b * n_r + i] = (float)ci;
    }
  }
}

// w[b][k] = sum_i T[k][i] c[b][i]: one warp per (b, k); FP32 products, lane
// partials reduced in FP64.
__global__ void wvec_kernel(const float *__restrict__ T,
                            const float *__restrict__ cvec, int n_bins,
                            int n_r, int kmin, int n_configs,
                            double *__restrict__ w) {
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (gw >= n_configs * n_bins) return;
  const int b = gw / n_bins, k = gw % n_bins;
  double acc = 0.0;
  if (k >= kmin) {
    const float *row = T + (size_t)k * n_r;
    const float *c = cvec + (size_t)b * n_r;
    float part = 0.f;
    for (int i = lane; i < n_r; i += 32) part = fmaf(row[i], c[i], part);
    acc = warp_sum((double)part);
  }
  if (lane == 0) w[(size_t)b * n_bins + k] = acc;
}

// Adjoint tables: tabs[b][sa][sb][m] = (A_kk, A_kk+1, B_kk, B_kk+1),
//   kk = 2m, k = kb0 + kk, W = 2 w_k f_sa f_sb / na_k (0 outside
//   [kmin, n_bins) or where na_k = 0), A = k W, B = W.
__global__ void adjoint_table_kernel(const double *__restrict__ w,
                                     const double *__restrict__ na,
                                     const float *__restrict__ ftab,
                                     int n_species, int n_bins, int kmin,
                                     int kb0, int kp, int n_configs,
                                     float4 *__restrict__ tabs) {
  const int kh = kp / 2;
  const size_t total = (size_t)n_configs * n_species * n_species * kh;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    const int m = idx % kh;
    size_t rest = idx / kh;
    const int sb = rest % n_species;
    rest /= n_species;
    const int sa = rest % n_species;
    const int b = (int)(rest / n_species);
    float A[2], B[2];
    for (int e = 0; e < 2; ++e) {
      const int k = kb0 + 2 * m + e;
      double W = 0.0;
      if (k >= kmin && k < n_bins) {
        const double nak = na[(size_t)b * n_bins + k];
        if (nak != 0.0)
          W = 2.0 * w[(size_t)b * n_bins + k] * (double)ftab[sa * n_bins + k] *
              (double)ftab[sb * n_bins + k] / nak;
      }
      A[e] = (float)((double)k * W);
      B[e] = (float)W;
    }
    tabs[(((size_t)b * n_species + sa) * n_species + sb) * kh + m] =
        make_float4(A[0], A[1], B[0], B[1]);
  }
}

// dF coefficient table for the reference-convention gradient:
//   coef[b][sa][sb][k] = -f_sa f_sb / na_k   (float division as the reference)
__global__ void gradfq_coef_kernel(const double *__restrict__ na,
                                   const float *__restrict__ ftab,
                                   int n_species, int n_bins, int n_configs,
                                   float *__restrict__ coef) {
  const size_t total = (size_t)n_configs * n_species * n_species * n_bins;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    const int k = idx % n_bins;
    size_t rest = idx / n_bins;
    const int sb = rest % n_species;
    rest /= n_species;
    const int sa = rest % n_species;
    const int b = (int)(rest / n_species);
    const float nak = (float)na[(size_t)b * n_bins + k];
    coef[idx] = -(ftab[sa * n_bins + k] * ftab[sb * n_bins + k]) / nak;
  }
}

// Compat potential gradient from an explicit grad_pdf: one warp per row,
// grad[row] = sum_i c_i gpdf[row][i], with c recomputed from (gcalc, gobs).
__global__ void potential_grad_rows_kernel(const double *__restrict__ gpdf,
                                           const float *__restrict__ cvec,
                                           int n_rows, int n_r,
                                           double *__restrict__ grad) {
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (gw >= n_rows) return;
  const double *row = gpdf + (size_t)gw * n_r;
  double acc = 0.0;
  for (int i = lane; i < n_r; i += 32) acc += (double)cvec[i] * row[i];
  acc = warp_sum(acc);
  if (lane == 0) grad[gw] = acc;
}

}  // namespace pyiid
