/*
 * debye_ref.c -- C restatements of pyIID's scattering path (TEST INFRASTRUCTURE).
 *
 * Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py
 * load this library; the pyiid_gb300 product never does.
 *
 * Two families:
 *   oracle_*  FP64 restatement of the reference formulas (exact values the
 *             reference's float32 code approximates), OpenMP over atoms/bins,
 *             for sizes the NumPy oracle cannot reach (sampled bins / rows).
 *   port_*    FP32 loop-for-loop port of the reference's default CPU path
 *             ('CPU' processor, kernel_type 'flat'):
 *               cpu_wrappers/flat_multi_cpu_wrap.py:22-134 (task split, sums),
 *               atomics/cpu_atomics.py:10-102 (allocation formulas, tasks),
 *               kernels/cpu_flat.py:16-194 (d, r, norm, omega, grad kernels),
 *               kernels/cpu_experimental.py:8-15 (gradient scatter),
 *               kernels/__init__.py:15-19 (k -> (i, j)).
 *             Each task materialises its [m, K] / [m, 3, K] float32 arrays
 *             and an [n, 3, K] result exactly as the numba code does; tasks
 *             run one per OpenMP thread instead of one per Pool process.
 *             numba itself is not installed, so this port is the timed
 *             stand-in for the reference CPU implementation.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------ FP64 oracle */

/* S_k for the requested bins: sum_{a>b} f_a f_b sin(Q_k r)/r, Q_k = k*qbin.
 * pos float32 [n][3], species [n], ftab [S][K].  Each bin's sum over the
 * rows a is split across the threads (a handful of bins at 20,000 atoms
 * still uses every core). */
void oracle_pair_sums(const float *pos, const int32_t *species, int n,
                      const float *ftab, int n_bins, double qbin,
                      const int32_t *bins, int nb, double *out) {
  for (int ib = 0; ib < nb; ++ib) {
    const int k = bins[ib];
    const double Q = (double)k * qbin;
    double s = 0.0;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : s)
    for (int a = 1; a < n; ++a) {
      const double fa = ftab[(size_t)species[a] * n_bins + k];
      double sa = 0.0;
      for (int b = 0; b < a; ++b) {
        const double dx = (double)pos[3 * a] - pos[3 * b];
        const double dy = (double)pos[3 * a + 1] - pos[3 * b + 1];
        const double dz = (double)pos[3 * a + 2] - pos[3 * b + 2];
        const double r = sqrt(dx * dx + dy * dy + dz * dz);
        sa += ftab[(size_t)species[b] * n_bins + k] * sin(Q * r) / r;
      }
      s += fa * sa;
    }
    out[ib] = s;
  }
}

/* True gradient rows dS_k/dx_a (without the normalisation) for the requested
 * atoms, all bins: out[ia][3][K]. */
void oracle_grad_rows(const float *pos, const int32_t *species, int n,
                      const float *ftab, int n_bins, double qbin,
                      const int32_t *atoms, int na, double *out) {
#pragma omp parallel for schedule(dynamic, 1)
  for (int ia = 0; ia < na; ++ia) {
    const int a = atoms[ia];
    double *o = out + (size_t)ia * 3 * n_bins;
    memset(o, 0, sizeof(double) * 3 * n_bins);
    for (int b = 0; b < n; ++b) {
      if (b == a) continue;
      const double dx = (double)pos[3 * a] - pos[3 * b];
      const double dy = (double)pos[3 * a + 1] - pos[3 * b + 1];
      const double dz = (double)pos[3 * a + 2] - pos[3 * b + 2];
      const double r = sqrt(dx * dx + dy * dy + dz * dz);
      const float *fa = ftab + (size_t)species[a] * n_bins;
      const float *fb = ftab + (size_t)species[b] * n_bins;
      for (int k = 0; k < n_bins; ++k) {
        const double Q = (double)k * qbin;
        const double g = (Q * cos(Q * r) - sin(Q * r) / r) / (r * r) *
                         (double)fa[k] * (double)fb[k];
        o[k] += g * dx;
        o[n_bins + k] += g * dy;
        o[2 * n_bins + k] += g * dz;
      }
    }
  }
}

/* --------------------------------------------------- FP32 reference port */

/* kernels/__init__.py:15-19 */
static void k_to_ij(long k, int *i, int *j) {
  double fi = floor((1.0 + sqrt(1.0 + 8.0 * (double)k)) / 2.0);
  *i = (int)fi;
  *j = (int)((double)k - fi * (fi - 1.0) / 2.0);
}

/* atoms/cpu_atomics.py:10-32 and :35-57 */
long port_fq_allocation(long n, long sv, double mem) {
  return (long)floor((0.8 * mem - 4.0 * sv * n - 12.0 * n) / (4.0 * (3 * sv + 4)));
}
long port_grad_allocation(long n, long qmax_bin, double mem) {
  return (long)floor((0.8 * mem - 16.0 * qmax_bin * n - 12.0 * n) /
                     (16.0 * (2 * qmax_bin + 1)));
}

/* One atomic_fq task (atoms/cpu_atomics.py:60-78): pairs [k_cov, k_cov+m). */
static void port_atomic_fq(const float *q, const float *scat, int n, int K,
                           float qbin, long m, long k_cov, double *res) {
  float *d = (float *)calloc((size_t)m * 3, sizeof(float));
  float *r = (float *)calloc((size_t)m, sizeof(float));
  float *norm = (float *)calloc((size_t)m * K, sizeof(float));
  float *omega = (float *)calloc((size_t)m * K, sizeof(float));
  float *fq = (float *)calloc((size_t)m * K, sizeof(float));
  for (long k = 0; k < m; ++k) { /* get_d_array cpu_flat.py:16-32 */
    int i, j;
    k_to_ij(k + k_cov, &i, &j);
    for (int w = 0; w < 3; ++w) d[k * 3 + w] = q[3 * i + w] - q[3 * j + w];
  }
  for (long k = 0; k < m; ++k) { /* get_r_array :37-52 */
    float t = 0.f;
    for (int w = 0; w < 3; ++w) t += d[k * 3 + w] * d[k * 3 + w];
    r[k] = sqrtf(t);
  }
  for (long k = 0; k < m; ++k) { /* get_normalization_array :57-74 */
    int i, j;
    k_to_ij(k + k_cov, &i, &j);
    for (int x = 0; x < K; ++x)
      norm[k * K + x] = scat[(size_t)i * K + x] * scat[(size_t)j * K + x];
  }
  for (int x = 0; x < K; ++x) { /* get_omega :79-96 */
    const float sv = qbin * (float)x;
    for (long k = 0; k < m; ++k) omega[k * K + x] = sinf(sv * r[k]) / r[k];
  }
  for (int x = 0; x < K; ++x) /* get_fq :101-104 */
    for (long k = 0; k < m; ++k) fq[k * K + x] = norm[k * K + x] * omega[k * K + x];
  for (int x = 0; x < K; ++x) res[x] = 0.0; /* fq.sum(axis=0, dtype=f64) */
  for (long k = 0; k < m; ++k)
    for (int x = 0; x < K; ++x) res[x] += (double)fq[k * K + x];
  free(d); free(r); free(norm); free(omega); free(fq);
}

/* One atomic_grad_fq task (atoms/cpu_atomics.py:81-102).  The task's
 * contributions are added into rtn [n][3][K]; the reference zeroes a fresh
 * [n,3,K] array per task and the parent sums them all, the port keeps one
 * array per thread and sums once (cheaper, i.e. favourable to the reference). */
static void port_atomic_grad(const float *q, const float *scat, int n, int K,
                             float qbin, long m, long k_cov, float *rtn) {
  float *d = (float *)malloc((size_t)m * 3 * sizeof(float));
  float *r = (float *)malloc((size_t)m * sizeof(float));
  float *norm = (float *)malloc((size_t)m * K * sizeof(float));
  float *omega = (float *)calloc((size_t)m * K, sizeof(float));
  float *gomega = (float *)calloc((size_t)m * 3 * K, sizeof(float));
  float *grad = (float *)malloc((size_t)m * 3 * K * sizeof(float));
  for (long k = 0; k < m; ++k) {
    int i, j;
    k_to_ij(k + k_cov, &i, &j);
    for (int w = 0; w < 3; ++w) d[k * 3 + w] = q[3 * i + w] - q[3 * j + w];
  }
  for (long k = 0; k < m; ++k) {
    float t = 0.f;
    for (int w = 0; w < 3; ++w) t += d[k * 3 + w] * d[k * 3 + w];
    r[k] = sqrtf(t);
  }
  for (long k = 0; k < m; ++k) {
    int i, j;
    k_to_ij(k + k_cov, &i, &j);
    for (int x = 0; x < K; ++x)
      norm[k * K + x] = scat[(size_t)i * K + x] * scat[(size_t)j * K + x];
  }
  for (int x = 0; x < K; ++x) {
    const float sv = qbin * (float)x;
    for (long k = 0; k < m; ++k) omega[k * K + x] = sinf(sv * r[k]) / r[k];
  }
  for (int x = 0; x < K; ++x) { /* get_grad_omega cpu_flat.py:122-131 */
    const float sv = (float)x * qbin;
    for (long k = 0; k < m; ++k) {
      const float rk = r[k];
      float a = sv * cosf(sv * rk) - omega[k * K + x];
      a /= rk * rk;
      for (int w = 0; w < 3; ++w) gomega[(k * 3 + w) * K + x] = a * d[k * 3 + w];
    }
  }
  for (long k = 0; k < m; ++k) /* get_grad_fq :136-156 */
    for (int w = 0; w < 3; ++w)
      for (int x = 0; x < K; ++x)
        grad[(k * 3 + w) * K + x] = norm[k * K + x] * gomega[(k * 3 + w) * K + x];
  for (long k = 0; k < m; ++k) { /* experimental_sum_grad_cpu */
    int i, j;
    k_to_ij(k + k_cov, &i, &j);
    for (int x = 0; x < K; ++x)
      for (int w = 0; w < 3; ++w) {
        rtn[((size_t)i * 3 + w) * K + x] -= grad[(k * 3 + w) * K + x];
        rtn[((size_t)j * 3 + w) * K + x] += grad[(k * 3 + w) * K + x];
      }
  }
  free(d); free(r); free(norm); free(omega); free(gomega); free(grad);
}

/* Runs tasks of `chunk` pairs covering pairs [0, n_pairs) (n_pairs <= the
 * configuration's n(n-1)/2), one task per thread at a time, and reduces them
 * as flat_multi_cpu_wrap.wrap_fq / wrap_fq_grad do before normalisation:
 *   sums[K]       = sum over tasks of the FP64 task sums   (may be NULL)
 *   grad[n][3][K] = sum over tasks of the task arrays      (may be NULL)
 * Returns the number of threads used. */
int port_fq_grad_tasks(const float *q, const float *scat, int n, int K,
                       double qbin_d, long chunk, long n_pairs, double *sums,
                       float *grad, int n_threads) {
  const float qbin = (float)qbin_d;
  const long n_tasks = (n_pairs + chunk - 1) / chunk;
  int used = 1;
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
  if (sums) memset(sums, 0, sizeof(double) * K);
  if (grad) memset(grad, 0, sizeof(float) * (size_t)n * 3 * K);
#pragma omp parallel
  {
#ifdef _OPENMP
#pragma omp single
    used = omp_get_num_threads();
#endif
    double *tsum = sums ? (double *)calloc(K, sizeof(double)) : NULL;
    double *res = sums ? (double *)malloc(sizeof(double) * K) : NULL;
    float *rtn = grad ? (float *)calloc((size_t)n * 3 * K, sizeof(float)) : NULL;
#pragma omp for schedule(dynamic, 1)
    for (long t = 0; t < n_tasks; ++t) {
      const long k_cov = t * chunk;
      const long m = (k_cov + chunk <= n_pairs) ? chunk : n_pairs - k_cov;
      if (sums) {
        port_atomic_fq(q, scat, n, K, qbin, m, k_cov, res);
        for (int x = 0; x < K; ++x) tsum[x] += res[x];
      }
      if (grad) port_atomic_grad(q, scat, n, K, qbin, m, k_cov, rtn);
    }
    if (sums) {
#pragma omp critical
      for (int x = 0; x < K; ++x) sums[x] += tsum[x];
    }
    if (grad) {
#pragma omp critical
      for (size_t i = 0; i < (size_t)n * 3 * K; ++i) grad[i] += rtn[i];
    }
    free(tsum); free(res); free(rtn);
  }
  return used;
}
