// spring_kernels.cuh -- spring potentials of pyiid/calc/spring_calc.py:
// spring_nrg / spring_force :99-144, voxel and atomwise energies :145-184,
// the centre-of-mass spring :185-251 and the attractive spring :252-331.
//
// Pair springs (ordered pairs i != j, d_ij = q_j - q_i, r = |d_ij|, FP32 as
// the reference's nxn kernels form them):
//   'rep' (type 0): active for r < rt,  'att' (type 1): active for r > rt,
//   energy = sum_{ordered, active} k (r - rt)^2 / 2,
//   force_i = sum_{j active} d_ij / r_ij * k (r_ij - rt)
// (the reference's forces, i.e. half of -dE/dq), NaN components -> 0.
// Atomwise energies (the energy change on removing atom i, the reference's
// calculate_atomwise_energy): -2 sum_j k (r_ij - rt)^2 / 2 over j != i with
// r <= rt (rep) or r >= rt (att).
// Centre-of-mass spring (type 2): per atom disp = q - com, dist = |disp|,
// active for dist > rt: energy k (dist - rt)^2 / 2, force -disp/dist k
// (dist - rt); its atomwise value is the reference's scalar
// 2 sum_i k (dist - rt)^2 / 2 over dist >= rt.
// Voxel energies (the energy change on inserting an atom at each voxel
// centre ((i + 1/2) res, (j + 1/2) res, (k + 1/2) res)): twice the sum of
// k (t - rt)^2 / 2 over atoms at distance t with t < rt (rep), t > rt (att),
// or of the centre's distance to com (com).
#pragma once

#include <cuda_runtime.h>

#include "transform_kernels.cuh"

namespace pyiid {

constexpr int kSpringBlock = 128;

__device__ __forceinline__ bool spring_active(int type, float r, float rt) {
  return type == 0 ? (r < rt) : (r > rt);
}

// One thread per atom i; positions of all atoms stream through shared memory
// in tiles of kSpringBlock.  Per-CTA energy partial (FP64) in part[blockIdx].
__global__ void __launch_bounds__(kSpringBlock)
    spring_pair_kernel(const float *__restrict__ pos, int n, float k,
                       float rt, int type, double *__restrict__ part,
                       float *__restrict__ forces,
                       double *__restrict__ atomwise) {
  __shared__ float3 sq[kSpringBlock];
  __shared__ double scratch[32];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float3 qi = make_float3(0.f, 0.f, 0.f);
  if (i < n) qi = make_float3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
  float e = 0.f, aw = 0.f, fx = 0.f, fy = 0.f, fz = 0.f;
  for (int j0 = 0; j0 < n; j0 += kSpringBlock) {
    __syncthreads();
    const int jl = j0 + threadIdx.x;
    if (jl < n)
      sq[threadIdx.x] = make_float3(pos[3 * jl], pos[3 * jl + 1],
                                    pos[3 * jl + 2]);
    __syncthreads();
    if (i >= n) continue;
    const int jn = min(kSpringBlock, n - j0);
    for (int jj = 0; jj < jn; ++jj) {
      const int j = j0 + jj;
      if (j == i) continue;
      const float dx = __fsub_rn(sq[jj].x, qi.x);
      const float dy = __fsub_rn(sq[jj].y, qi.y);
      const float dz = __fsub_rn(sq[jj].z, qi.z);
      const float r = __fsqrt_rn(__fmaf_rn(dx, dx, __fmaf_rn(dy, dy, dz * dz)));
      const float x = r - rt;
      const float m = k * x;
      if (spring_active(type, r, rt)) {
        e = fmaf(0.5f * m, x, e);
        const float ir = 1.0f / r;
        const float gx = dx * ir * m, gy = dy * ir * m, gz = dz * ir * m;
        fx += isnan(gx) ? 0.f : gx;
        fy += isnan(gy) ? 0.f : gy;
        fz += isnan(gz) ? 0.f : gz;
      }
      if (type == 0 ? (r <= rt) : (r >= rt)) aw = fmaf(m, x, aw);
    }
  }
  if (i < n) {
    if (forces) {
      forces[3 * i] = fx;
      forces[3 * i + 1] = fy;
      forces[3 * i + 2] = fz;
    }
    if (atomwise) atomwise[i] = -(double)aw;
  }
  double v[1] = {(double)e};
  block_sum<1>(v, scratch);
  if (threadIdx.x == 0) part[blockIdx.x] = v[0];
}

// Centre-of-mass spring, one thread per atom (same outputs as above; the
// atomwise scalar goes to apart[blockIdx] and is summed with the energy).
__global__ void __launch_bounds__(kSpringBlock)
    com_spring_kernel(const float *__restrict__ pos, int n, float k,
                      float rt, double cx, double cy, double cz,
                      double *__restrict__ part, double *__restrict__ apart,
                      float *__restrict__ forces) {
  __shared__ double scratch[64];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double e = 0.0, aw = 0.0;
  if (i < n) {
    const double dx = (double)pos[3 * i] - cx;
    const double dy = (double)pos[3 * i + 1] - cy;
    const double dz = (double)pos[3 * i + 2] - cz;
    const float dist = (float)sqrt(dx * dx + dy * dy + dz * dz);
    const float x = dist - rt;
    float f[3] = {0.f, 0.f, 0.f};
    if (dist > rt) {
      e = 0.5 * (double)(k * x) * (double)x;
      const float m = k * x;
      f[0] = -(float)dx / dist * m;
      f[1] = -(float)dy / dist * m;
      f[2] = -(float)dz / dist * m;
    }
    if (dist >= rt) aw = (double)(k * x) * (double)x;
    if (forces) {
      forces[3 * i] = f[0];
      forces[3 * i + 1] = f[1];
      forces[3 * i + 2] = f[2];
    }
  }
  double v[2] = {e, aw};
  block_sum<2>(v, scratch);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = v[0];
    apart[blockIdx.x] = v[1];
  }
}

// Sum of n per-CTA partials in a fixed order (one CTA).
__global__ void sum_partials_kernel(const double *__restrict__ part, int n,
                                    double *__restrict__ out) {
  __shared__ double scratch[32];
  double v[1] = {0.0};
  for (int i = threadIdx.x; i < n; i += blockDim.x) v[0] += part[i];
  block_sum<1>(v, scratch);
  if (threadIdx.x == 0) *out = v[0];
}

// Voxel energies, one thread per voxel.
__global__ void __launch_bounds__(kSpringBlock)
    spring_voxel_kernel(const float *__restrict__ pos, int n, float k,
                        float rt, int type, double cx, double cy, double cz,
                        int nx, int ny, int nz, float res,
                        double *__restrict__ voxels) {
  __shared__ float3 sq[kSpringBlock];
  const long long nv = (long long)nx * ny * nz;
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int iz = (int)(v % nz), iy = (int)((v / nz) % ny),
            ix = (int)(v / ((long long)nz * ny));
  const float x = ((float)ix + 0.5f) * res, y = ((float)iy + 0.5f) * res,
              z = ((float)iz + 0.5f) * res;
  float acc = 0.f;
  if (type == 2) {
    if (v < nv) {
      const double dx = x - cx, dy = y - cy, dz = z - cz;
      const float t = (float)sqrt(dx * dx + dy * dy + dz * dz);
      if (t > rt) acc = 0.5f * k * (t - rt) * (t - rt);
    }
  } else {
    for (int j0 = 0; j0 < n; j0 += kSpringBlock) {
      __syncthreads();
      const int jl = j0 + threadIdx.x;
      if (jl < n)
        sq[threadIdx.x] = make_float3(pos[3 * jl], pos[3 * jl + 1],
                                      pos[3 * jl + 2]);
      __syncthreads();
      if (v >= nv) continue;
      const int jn = min(kSpringBlock, n - j0);
      for (int jj = 0; jj < jn; ++jj) {
        const float dx = x - sq[jj].x, dy = y - sq[jj].y, dz = z - sq[jj].z;
        const float t =
            __fsqrt_rn(__fmaf_rn(dx, dx, __fmaf_rn(dy, dy, dz * dz)));
        if (spring_active(type, t, rt)) acc = fmaf(0.5f * k * (t - rt), t - rt, acc);
      }
    }
  }
  if (v < nv) voxels[v] = 2.0 * (double)acc;
}

}  // namespace pyiid
