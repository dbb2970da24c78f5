/*
 * pyiid_gb300.h -- C ABI of the GB300 (sm_103a) elastic-scattering library.
 *
 * The library evaluates the Debye scattering chain of pyIID on one GPU:
 *
 *   pair distances r_ab -> F(Q) = 2 * sum_{a>b} f_a f_b sin(Q r_ab)/r_ab / na(Q)
 *   F(Q) -> G(r) (the reference's FFT transform, as an exact linear map)
 *   G(r) -> Rw or chi^2 against an observed G(r), and the position gradient.
 *
 * Conventions shared by every entry point
 *   - All functions return an int status (PYIID_OK == 0).  On failure the
 *     message is available from pyiid_last_error(ctx) (or pyiid_last_error(NULL)
 *     when no context exists yet).  Nothing aborts the process.
 *   - Pointers documented "device" must be CUDA device (or managed) memory of
 *     the context's device.  Pointers documented "host" are read during the
 *     call and may be freed afterwards.
 *   - Work is enqueued on the context's stream (pyiid_set_stream) and is
 *     asynchronous with respect to the host unless stated otherwise.
 *   - Q grids are uniform and start at zero: Q_k = k * qbin, k in [0, n_bins).
 *     Output bins below k_begin are written as zero and never computed.
 *   - Atoms carry a species id; per-species form factors f_s(Q_k) are given as
 *     a host table [n_species][n_bins] (the reference's per-atom
 *     'F(Q) scatter' / 'PDF scatter' arrays have one distinct row per species).
 *   - Numerical semantics follow the reference: NaN results (coincident atoms,
 *     fewer than two atoms) become 0 and +-inf become +-FLT_MAX, as numpy's
 *     nan_to_num does on the reference's float32 arrays.
 *
 * One context per host thread / stream.  Contexts are independent; the only
 * shared state is read-only.
 */
#ifndef PYIID_GB300_H
#define PYIID_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  PYIID_OK = 0,
  PYIID_ERR_INVALID_ARG = 1,
  PYIID_ERR_CUDA = 2,
  PYIID_ERR_OOM = 3,
  PYIID_ERR_DEVICE_FLAG = 4,
  PYIID_ERR_TIMEOUT = 5
};

enum { PYIID_POTENTIAL_RW = 0, PYIID_POTENTIAL_CHI_SQ = 1 };

typedef struct pyiid_ctx pyiid_ctx;

/* Library version as MAJOR*10000 + MINOR*100 + PATCH. */
int pyiid_version(void);

/* Create a context bound to CUDA device `device` (the default stream is used
 * until pyiid_set_stream is called).  Replaces the processor probe of
 * pyiid/experiments/elasticscatter/__init__.py:29-38 (check_gpu) and the
 * per-GPU context handling of gpu_wrappers/gpu_wrap.py:287-314. */
int pyiid_create(pyiid_ctx **out, int device);
int pyiid_destroy(pyiid_ctx *ctx);

/* Enqueue subsequent work on `stream` (a cudaStream_t; NULL = legacy default). */
int pyiid_set_stream(pyiid_ctx *ctx, void *stream);

/* Wait for all work enqueued by this context.  Returns PYIID_ERR_TIMEOUT
 * (and clears the condition) when a kernel launched since the last call
 * gave up one of its bounded waits on its own pipeline (the tensor-core
 * G(r) gradient of pyiid_grad_pdf); that kernel's output is then invalid. */
int pyiid_synchronize(pyiid_ctx *ctx);

/* Last error message of `ctx` (or of the last failed pyiid_create when ctx is
 * NULL).  The string stays valid until the next call on the same context. */
const char *pyiid_last_error(const pyiid_ctx *ctx);

/* Number of kernels this context has launched so far (for launch accounting). */
int64_t pyiid_launch_count(const pyiid_ctx *ctx);

/* ------------------------------------------------------------------------ *
 * Reduced structure factor.
 *
 * fq[k] = 2 * nan_to_num( S_k / na_k ),  k in [k_begin, n_bins)
 *   S_k  = sum_{a>b} f_a(Q_k) f_b(Q_k) sin(Q_k r_ab) / r_ab
 *   na_k = n_atoms * mean_{a>b} f_a(Q_k) f_b(Q_k)
 * Pair sums are accumulated in FP32 (compensated) per tile and reduced in FP64.
 *
 * Replaces wrap_fq of cpu_wrappers/flat_multi_cpu_wrap.py:22-60 (same value as
 * cpu_wrappers/flat_serial_cpu_wrap.py:13-69, cpu_wrappers/nxn_cpu_wrap.py:9-69
 * and gpu_wrappers/gpu_wrap.py:119-156), i.e. the `self.fq` plug-in of
 * ElasticScatter (elasticscatter/__init__.py:101, 254, 277).
 *   positions : device float [n_atoms][3]
 *   species   : host int32 [n_atoms], values in [0, n_species)
 *   scatter   : host float [n_species][n_bins]
 *   fq        : device float [n_bins]
 * ------------------------------------------------------------------------ */
int pyiid_fq(pyiid_ctx *ctx, const float *positions, const int32_t *species,
             int n_atoms, const float *scatter, int n_species, int n_bins,
             double qbin, int k_begin, float *fq);

/* F(Q) of many configurations in one pass (one pair-sum launch over the
 * work items of every configuration, then one finishing launch).
 * Configuration b owns atoms offsets[b] .. offsets[b+1]-1 of the packed
 * positions/species; all share one Q grid and one species table.
 *   positions : device float [total_atoms][3]
 *   species   : host int32   [total_atoms]
 *   offsets   : host int32   [n_configs + 1]
 *   fq        : device float [n_configs][n_bins]
 * Replaces a Python loop of wrap_fq calls (flat_multi_cpu_wrap.py:22-60), one
 * per configuration. */
int pyiid_batch_fq(pyiid_ctx *ctx, const float *positions,
                   const int32_t *species, const int32_t *offsets,
                   int n_configs, const float *scatter, int n_species,
                   int n_bins, double qbin, int k_begin, float *fq);

/* Gradient of F(Q) in the reference's convention:
 *   grad[a][c][k] = -(1/na_k) * d S_k / d x_{a,c}  ( = -1/2 * dF_k/dx_{a,c} ),
 * k in [k_begin, n_bins), NaN -> 0 per element as the reference does.
 * Replaces wrap_fq_grad of cpu_wrappers/flat_multi_cpu_wrap.py:63-102 (and
 * flat_serial_cpu_wrap.py:72-133, nxn_cpu_wrap.py:72-137,
 * gpu_wrappers/gpu_wrap.py:159-194), the `self.grad` plug-in.
 *   grad : device float [n_atoms][3][n_bins] */
int pyiid_grad_fq(pyiid_ctx *ctx, const float *positions,
                  const int32_t *species, int n_atoms, const float *scatter,
                  int n_species, int n_bins, double qbin, int k_begin,
                  float *grad);

/* F(Q) and its gradient from one pass over the pairs: fq as pyiid_fq and
 * grad as pyiid_grad_fq return them (same conventions, same tolerances; the
 * pair terms are summed in a different order).  The gradient kernel already
 * generates sin(Q_k r) for every ordered pair and bin, so F(Q) costs one
 * more packed FMA per two bins instead of a second pass.  Replaces the
 * get_fq + get_grad_fq pair of calls a calculator makes on one
 * configuration (elasticscatter/__init__.py:304-341 and :477-496).
 *   fq   : float [n_bins]
 *   grad : float [n_atoms][3][n_bins]
 * Both outputs may be device memory or pinned host memory mapped into the
 * device (cudaHostAlloc / cudaHostRegister): the kernel then stores the
 * results over the host link while it computes, so no separate
 * device-to-host copy follows (zero-copy).  Other pointers are rejected. */
int pyiid_fq_grad(pyiid_ctx *ctx, const float *positions,
                  const int32_t *species, int n_atoms, const float *scatter,
                  int n_species, int n_bins, double qbin, int k_begin,
                  float *fq, float *grad);

/* One configuration split across processes (one per GPU, e.g. a single
 * large particle): the species-sorted atom tiles are cut into n_parts
 * contiguous ranges of nearly equal work, and part `part` evaluates the
 * pairs its tiles own in one pass (as pyiid_fq_grad):
 *   sums : device double [n_bins]  raw Debye sums S_k of its pairs (0 for
 *          k < k_begin); add them over the parts (one all-reduce of K
 *          doubles) and pass the total to pyiid_fq_from_sums for F(Q);
 *   grad : device float [n_atoms][3][n_bins]: the complete gradient rows of
 *          its atoms (each part sweeps all atoms for its rows); rows of
 *          other parts are left untouched, so no gradient exchange is needed;
 *   rows : host int32 [n_atoms] or NULL: 1 for the atoms whose rows it wrote.
 * The parts' rows partition the atoms.  Has no reference counterpart (the
 * reference's multi-GPU farm splits pair chunks and sums [N][3][K] arrays on
 * the host, gpu_wrappers/gpu_wrap.py:287-314). */
int pyiid_fq_grad_part(pyiid_ctx *ctx, const float *positions,
                       const int32_t *species, int n_atoms,
                       const float *scatter, int n_species, int n_bins,
                       double qbin, int k_begin, int part, int n_parts,
                       double *sums, float *grad, int32_t *rows);

/* F(Q) [n_bins] (device float) from the summed raw sums of all parts:
 * F_k = 2 nan_to_num(S_k / na_k) for k >= k_begin, 0 below. */
int pyiid_fq_from_sums(pyiid_ctx *ctx, const int32_t *species, int n_atoms,
                       const float *scatter, int n_species, int n_bins,
                       int k_begin, const double *sums, float *fq);

/* ------------------------------------------------------------------------ *
 * F(Q) -> G(r).
 *
 * gr[i] = sum_k F'_k T_k(rgrid[i]) where F' is fq with bins below
 * ceil(qmin/qstep) set to zero and T is the linear map equal to the
 * reference's zero-padded odd-extension FFT followed by linear interpolation
 * (kernels/master_kernel.py:39-203, get_pdf_at_qmin / fft_fq_to_gr /
 * fft_gr_to_fq).  T is built once per (qstep, rstep, qmin, rgrid, n_bins) on
 * the host in FP64 and cached on the device.
 *   fq    : device float  [n_configs][n_bins]   (bins from Q = 0)
 *   rgrid : host double   [n_r]
 *   gr    : device double [n_configs][n_r]
 * Replaces get_pdf_at_qmin (kernels/master_kernel.py:39-105). */
int pyiid_pdf(pyiid_ctx *ctx, const float *fq, int n_configs, int n_bins,
              double qstep, double rstep, const double *rgrid, int n_r,
              double qmin, double *gr);

/* Gradient of G(r): the same map applied to each of the 3N rows of a
 * reference-convention grad_fq.
 *   grad_fq  : device float  [n_atoms][3][n_bins]
 *   grad_pdf : device double [n_atoms][3][n_r]   (every element written)
 * On the tensor cores: rows scaled by powers of two and split into two FP16
 * halves, three products with FP32 accumulation; relative error ~1.2e-6 of
 * the FP64 product.
 * Replaces grad_pdf of kernels/master_kernel.py:276-290 and
 * gpu_wrappers/gpu_wrap.py:197-284 (the `self.grad_pdf` plug-in). */
int pyiid_grad_pdf(pyiid_ctx *ctx, const float *grad_fq, int n_atoms,
                   int n_bins, double qstep, double rstep, const double *rgrid,
                   int n_r, double qmin, double *grad_pdf);

/* ------------------------------------------------------------------------ *
 * Potentials.
 *
 * out[0] = Rw (or chi^2), out[1] = scale, for each of n_configs rows; the
 * branch for a non-positive scale is the reference's (Rw = 1, scale = 1;
 * chi^2 uses scale = 1).
 *   gobs  : device double [n_r] (shared by all configs)
 *   gcalc : device double [n_configs][n_r]
 *   out   : device double [n_configs][2]
 * Replaces get_rw / get_chi_sq / get_scale (kernels/master_kernel.py:206-266,
 * 388-389) behind wrap_rw / wrap_chi_sq (calc/__init__.py:10-53). */
int pyiid_potential(pyiid_ctx *ctx, const double *gobs, const double *gcalc,
                    int n_configs, int n_r, int potential, double *out);

/* Rw with per-point weights, get_rw(gobs, gcalc, weight) of
 * kernels/master_kernel.py:206-236:
 *   a = (gcalc.gobs)/(gcalc.gcalc) (unweighted, get_scale :388-389);
 *   a <= 0 -> (Rw, scale) = (1, 1);
 *   else Rw = sqrt(sum_i w_i (gobs_i - a gcalc_i)^2 / sum_i w_i gobs_i^2).
 *   weight : device double [n_r]; other arguments as pyiid_potential
 *            (out[2 b] = Rw, out[2 b + 1] = scale). */
int pyiid_potential_weighted(pyiid_ctx *ctx, const double *gobs,
                             const double *gcalc, const double *weight,
                             int n_configs, int n_r, double *out);

/* Gradient of the potential from an explicit G(r) gradient:
 *   grad[a][c] = sum_r c_r * grad_pdf[a][c][r]  with the reference's c_r.
 *   grad_pdf : device double [n_atoms][3][n_r]
 *   grad     : device double [n_atoms][3]
 * Replaces get_grad_rw / get_grad_chi_sq / get_grad_scale
 * (kernels/master_kernel.py:293-376, 392-396) behind wrap_grad_rw /
 * wrap_grad_chi_sq (calc/__init__.py:56-105). */
int pyiid_potential_grad(pyiid_ctx *ctx, const double *grad_pdf,
                         const double *gcalc, const double *gobs, int n_atoms,
                         int n_r, int potential, double *grad);

/* ------------------------------------------------------------------------ *
 * Fused potential and adjoint gradient for a batch of configurations.
 *
 * For each configuration b (atoms offsets[b] .. offsets[b+1]-1 of the packed
 * arrays) computes on the PDF grid: F(Q) -> G(r) -> potential, and the exact
 * gradient d(potential)/d(positions) through the adjoint of the chain
 * (no [N,3,K] or [N,3,R] intermediate).  The gradient is the TRUE gradient
 * (the reference's Calc1D forces equal -1/2 * conv * this; see
 * calc/calc_1d.py:89-95 and cpu_experimental.py:8-15).
 *   positions : device float  [total_atoms][3]
 *   species   : host int32    [total_atoms]
 *   offsets   : host int32    [n_configs + 1]
 *   scatter   : host float    [n_species][n_bins]
 *   gobs      : device double [n_r]
 *   energy    : device double [n_configs][2]  (potential, scale)
 *   grad      : device float  [total_atoms][3]  (may be NULL: energy only)
 *   gcalc     : device double [n_configs][n_r]  (may be NULL)
 *   fq        : device float  [n_configs][n_bins] (may be NULL)
 * Replaces, for one configuration, the call chain of Calc1D.calculate
 * (calc/calc_1d.py:44-95) -> get_pdf / get_grad_pdf
 * (elasticscatter/__init__.py:343-391, 498-524) -> get_rw / get_grad_rw. */
int pyiid_batch_potential_grad(pyiid_ctx *ctx, const float *positions,
                               const int32_t *species, const int32_t *offsets,
                               int n_configs, const float *scatter,
                               int n_species, int n_bins, double qstep,
                               double rstep, const double *rgrid, int n_r,
                               double qmin, const double *gobs, int potential,
                               double *energy, float *grad, double *gcalc,
                               float *fq);

/* ------------------------------------------------------------------------ *
 * Single-atom Metropolis moves with O(N K) exact energy changes.
 *
 * A step proposes, for every chain (configuration), one atom and a Gaussian
 * displacement, computes the exact change of the Debye sums
 *   S_k = sum_{a>b} f_a(Q_k) f_b(Q_k) sin(Q_k r_ab) / r_ab   (PDF grid)
 * from the N-1 pair terms of that atom, the proposed F and potential V', and
 * accepts with probability min(1, exp(-conv (V' - V) / kT)).  This is the
 * exact energy difference the reference's Monte Carlo moves obtain by
 * re-evaluating the whole configuration (sim/gcmc.py:13-114 add_atom /
 * del_atom call get_potential_energy on a copy; sim/hmc.py:66-92 mh_accept),
 * at O(N K) instead of O(N^2 K) per proposal.  The potential is formed
 * without G(r): with the transform G = T^T F, u = F.(T gobs) and
 * q = F^T (T T^T) F give G.gobs and G.G, and ee = gobs.gobs - u^2 / q is
 * |gobs - s G|^2 at the optimal scale; the chain state keeps S, F, u, q and
 * ee, and a proposal F' = F + dF changes them by du = dF.(T gobs),
 * dq = dF^T (T T^T) (F + F') and ee' - ee = -[(2 u du + du^2) q - u^2 dq] /
 * (q (q + dq)), so that it costs K^2, not K R, and the acceptance test runs
 * in FP32 on increments.
 *
 * state (device double [pyiid_mh_state_size(n_configs, n_bins)]):
 *   v [n_bins] (T gobs), gobs.gobs, 1 / gobs.gobs, S [2][n_configs][n_bins],
 *   (u, q, ee, 0) [n_configs], F [2][n_configs][n_bins] as float32, then
 *   cur [n_configs] as int32: chain c's state is S[cur[c]][c], F[cur[c]][c]
 *   (the other buffer holds the last proposal).
 *
 * pyiid_mh_init: full exact evaluation of every chain into state and
 * energy (device double [n_configs][2]: V, scale); call it to start, when
 * gobs changes, and whenever positions were changed by anything else (it
 * also bounds the drift of the running sums).  Arguments as
 * pyiid_batch_potential_grad (scatter on the PDF grid).  The first call for a
 * grid builds T T^T on the device (n_bins^2 doubles, kept with T); at most
 * 3200 bins.
 *
 * pyiid_mh_steps: n_steps Metropolis steps of every chain, enqueued without
 * host synchronisation (3 kernels per step; capturable in a CUDA graph after
 * a first call with n_steps = 0 has sized the context's buffers).
 *   positions : device float [total][3], updated in place
 *   conv, kT  : energy = conv * V; kT > 0 in the same unit
 *   sigma     : displacement standard deviation per coordinate
 *   seed      : generator key.  Proposal t of chain c depends only on
 *               (seed, c, t): Philox4x32-10 counters (t, c, 0/1)
 *   state, energy : from pyiid_mh_init (updated)
 *   counter   : device uint64 [n_configs], proposals made so far per chain
 *               (start at 0; advanced by one per step)
 *   accepted  : device int64  [n_configs], incremented on acceptance
 *   trace     : device double [n_steps][n_configs][8] or NULL:
 *               atom (index within its configuration), proposed x, y, z,
 *               log u, V', accepted (0/1), V before the step
 * A proposal that makes two atoms coincide, or any NaN potential, is
 * rejected.  Chains with fewer than two atoms never move. */
size_t pyiid_mh_state_size(int n_configs, int n_bins);
int pyiid_mh_init(pyiid_ctx *ctx, const float *positions,
                  const int32_t *species, const int32_t *offsets,
                  int n_configs, const float *scatter, int n_species,
                  int n_bins, double qstep, double rstep, const double *rgrid,
                  int n_r, double qmin, const double *gobs, int potential,
                  double *state, double *energy);
int pyiid_mh_steps(pyiid_ctx *ctx, float *positions, const int32_t *species,
                   const int32_t *offsets, int n_configs, const float *scatter,
                   int n_species, int n_bins, double qstep, double rstep,
                   const double *rgrid, int n_r, double qmin, int potential,
                   double conv, double kT, float sigma, uint64_t seed,
                   int n_steps, double *state, double *energy,
                   uint64_t *counter, int64_t *accepted, double *trace);

/* Host-chosen moves with O(N K) exact energies (grand-canonical and other
 * Monte Carlo schemes whose proposals and acceptance live on the host, as in
 * the reference's sim/gcmc.py:13-114 add_atom / del_atom).
 *
 * pyiid_mc_propose: one proposal per chain, evaluated exactly without
 * changing the state; returns when eval is ready.
 *   mode        : host int32 [n_configs]: PYIID_MOVE_DISPLACE (atom moves to
 *                 xyz), PYIID_MOVE_INSERT (a new atom of species
 *                 new_species at xyz; the configuration must have >= 1
 *                 atom), PYIID_MOVE_REMOVE (atom deleted; >= 2 atoms)
 *   atom        : host int32 [n_configs], index within the configuration
 *   xyz         : host float [n_configs][3]
 *   new_species : host int32 [n_configs]
 *   state       : from pyiid_mh_init for the current configurations
 *   eval        : device double [n_configs][8]: V' (potential of the
 *                 proposed configuration), its scale, u', q', ee' (the Gram
 *                 scalars), V of the current state (0 if not tracked), 0, 0
 * Arguments otherwise as pyiid_mh_steps.  The normalisation na of an
 * inserted or removed atom's configuration is the one the layout of the
 * new configuration gives.
 *
 * pyiid_mc_accept: for chains with accept[c] != 0 the evaluated proposal
 * becomes the state (host int32 accept [n_configs]; eval from the last
 * pyiid_mc_propose; energy as pyiid_mh_init's).  The caller then applies the
 * move to its positions / species / offsets (for insertion and removal the
 * next call sees the new configuration sizes).  Returns when done. */
enum { PYIID_MOVE_DISPLACE = 0, PYIID_MOVE_INSERT = 1, PYIID_MOVE_REMOVE = 2 };
int pyiid_mc_propose(pyiid_ctx *ctx, const float *positions,
                     const int32_t *species, const int32_t *offsets,
                     int n_configs, const float *scatter, int n_species,
                     int n_bins, double qstep, double rstep,
                     const double *rgrid, int n_r, double qmin, int potential,
                     const int32_t *mode, const int32_t *atom,
                     const float *xyz, const int32_t *new_species,
                     double *state, double *eval);
int pyiid_mc_accept(pyiid_ctx *ctx, const int32_t *accept, int n_configs,
                    int n_bins, const double *eval, double *state,
                    double *energy);

/* ------------------------------------------------------------------------ *
 * Spring potentials (pyiid/calc/spring_calc.py), the pair potentials the
 * reference's samplers combine with the scattering potential (MultiCalc).
 *   sp_type : PYIID_SPRING_REP (pairs closer than rt, spring_nrg /
 *             spring_force :99-141), PYIID_SPRING_ATT (pairs farther than
 *             rt, att_spring_* :252-295), PYIID_SPRING_COM (atoms farther
 *             than rt from com, com_spring_* :185-217)
 *   com     : host double [3], the centre of mass (PYIID_SPRING_COM only)
 * pyiid_spring: energy (device double [1]) = sum over ordered pairs (or
 *   atoms) of k (r - rt)^2 / 2; forces (device float [n][3], may be NULL)
 *   are the reference's (half of -dE/dq for the pair springs); atomwise
 *   (device double, may be NULL) is calculate_atomwise_energy: per atom the
 *   energy change on its removal for the pair springs ([n]), and the
 *   reference's scalar for the com spring ([1]).
 * pyiid_spring_voxels: calculate_voxel_energy (voxel_spring_nrg :145-166 and
 *   its att/com twins): for each voxel centre ((i+1/2) res, (j+1/2) res,
 *   (k+1/2) res) the energy change on inserting an atom there; voxels is a
 *   device double [nx][ny][nz]. */
enum { PYIID_SPRING_REP = 0, PYIID_SPRING_ATT = 1, PYIID_SPRING_COM = 2 };
int pyiid_spring(pyiid_ctx *ctx, const float *positions, int n_atoms,
                 double k, double rt, int sp_type, const double *com,
                 double *energy, float *forces, double *atomwise);
int pyiid_spring_voxels(pyiid_ctx *ctx, const float *positions, int n_atoms,
                        double k, double rt, int sp_type, const double *com,
                        int nx, int ny, int nz, double resolution,
                        double *voxels);

/* F(Q) without device allocation.
 *
 * Same arguments, result and error behaviour as pyiid_fq, for callers that
 * cannot allocate device memory (a process whose device memory is owned by
 * another framework's pool, code inside a stream capture of a pre-sized
 * graph, hosts without a device allocator).  All device-side intermediates
 * live in one fixed 32 MiB device array inside the library, which every GPU
 * that loads the library holds until the process exits; the call performs no
 * cudaMalloc or cudaFree.  Problems whose intermediates exceed the array
 * (about 8 * n_bins bytes per work item, i.e. per pair of 32-atom tiles
 * spanning up to 32 tiles, plus small per-atom tables) are rejected with
 * PYIID_ERR_INVALID_ARG and a message naming the size needed.
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * The call returns when fq is ready (it synchronizes the context stream).
 * Every call reuses the same array and overwrites everything it reads, so
 * results never depend on earlier calls, but calls that overlap on the GPU
 * (other streams or threads) race on it: serialize them.
 * No counterpart in the reference (its processors allocate per call). */
int pyiid_fq_noalloc(pyiid_ctx *ctx, const float *positions,
                     const int32_t *species, int n_atoms, const float *scatter,
                     int n_species, int n_bins, double qbin, int k_begin,
                     float *fq);

/* ------------------------------------------------------------------------ *
 * Learned surrogate of the potential (first stage of delayed acceptance).
 *
 * No counterpart in the reference: these serve the delayed-acceptance
 * sampler that cheaply screens proposals before the exact Debye potential.
 *
 * Radial-basis descriptors of every atom of a packed batch:
 *   feat[a][c] = sum_{b != a, same configuration, r < r_cut}
 *                exp(-(r_ab - mu_c)^2 / (2 sigma^2)) (1 + cos(pi r_ab/r_cut))/2,
 *   mu_c = c r_cut / (n_centres - 1),  2 <= n_centres <= 64.
 *   positions : device float [total][3];  offsets : host int32 [n_configs+1]
 *   feat_bf16 : device bfloat16 [total][n_centres]
 *   feat_f32  : device float [total][n_centres] or NULL */
int pyiid_rbf_features(pyiid_ctx *ctx, const float *positions,
                       const int32_t *offsets, int n_configs, int n_centres,
                       float r_cut, float sigma, void *feat_bf16,
                       float *feat_f32);

/* Per-atom MLP  y_a = w3 . silu(W2^T silu(W1^T x_a + b1) + b2) + b3  summed
 * per configuration: energy[c] = sum_{a in c} y_a (FP64).  The two hidden
 * layers are BF16 tensor-core GEMMs with FP32 accumulation.
 *   feat_bf16 : device bf16 [n_atoms][n_in]
 *   w1_bf16   : device bf16 [n_in][n_hidden],  b1 : device float [n_hidden]
 *   w2_bf16   : device bf16 [n_hidden][n_hidden], b2 : device float [n_hidden]
 *   w3        : device float [n_hidden],       b3 : device float [1]
 *   energy    : device double [n_configs]
 * The activations are kept in the context for pyiid_mlp_backward. */
int pyiid_mlp_forward(pyiid_ctx *ctx, const void *feat_bf16, int n_atoms,
                      int n_in, const int32_t *offsets, int n_configs,
                      const void *w1_bf16, const float *b1,
                      const void *w2_bf16, const float *b2, const float *w3,
                      const float *b3, int n_hidden, double *energy);

/* Gradients of L with respect to the MLP parameters for the most recent
 * pyiid_mlp_forward on this context, given d_energy = dL/denergy (device
 * double [n_configs]).  Outputs are device float arrays shaped like the
 * parameters (overwritten). */
int pyiid_mlp_backward(pyiid_ctx *ctx, const double *d_energy, float *g_w1,
                       float *g_b1, float *g_w2, float *g_b2, float *g_w3,
                       float *g_b3);

/* Neighbour lists for the surrogate: for every atom a of a packed batch,
 * the atoms b != a of its configuration with |x_a - x_b| < r_list, in
 * increasing b.
 *   nbr_idx : device int32 [total][max_nb] (indices into the packed arrays)
 *   nbr_cnt : device int32 [total], the number of neighbours found; a count
 *             above max_nb means the list overflowed (only max_nb stored)
 * No counterpart in the reference. */
int pyiid_neighbor_list(pyiid_ctx *ctx, const float *positions,
                        const int32_t *offsets, int n_configs, float r_list,
                        int max_nb, int32_t *nbr_idx, int32_t *nbr_cnt);

/* Energy and forces of the surrogate for trajectories driven by it (the
 * cheap first stage of delayed-acceptance HMC).  From neighbour lists
 * (pyiid_neighbor_list with r_list >= r_cut) the descriptors of
 * pyiid_rbf_features, the MLP of pyiid_mlp_forward and its gradient with
 * respect to the descriptors (the same BF16 tensor-core GEMMs, transposed),
 * then per atom
 *   dE/dx_a = sum_{b in list(a), r_ab < r_cut} sum_c (dE/dfeat[a][c] +
 *             dE/dfeat[b][c]) dphi_c/dr (x_a - x_b) / r_ab.
 *   energy    : device double [n_configs], E = sum_a y_a (unscaled)
 *   forces    : device float [total][3] = -scale dE/dx, or NULL (energy
 *               only); forces need n_centres divisible by 8
 *   feat_bf16 : device bfloat16 [total][n_centres] for the descriptors, or
 *               NULL (context workspace)
 * Other arguments as pyiid_rbf_features / pyiid_mlp_forward.  Uses its own
 * workspace (training calls on the same context do not disturb it); after a
 * first call with the same sizes the call allocates nothing and can be
 * captured in a CUDA graph.  No counterpart in the reference. */
int pyiid_surrogate_forces(pyiid_ctx *ctx, const float *positions,
                           const int32_t *offsets, int n_configs,
                           const int32_t *nbr_idx, const int32_t *nbr_cnt,
                           int max_nb, int n_centres, float r_cut,
                           float sigma, const void *w1_bf16, const float *b1,
                           const void *w2_bf16, const float *b2,
                           const float *w3, const float *b3, int n_hidden,
                           float scale, double *energy, float *forces,
                           void *feat_bf16);

/* ------------------------------------------------------------------------ *
 * Launch-shape variants (autotuning).
 *
 * The pair kernels come in several launch shapes (bins per thread, pairs
 * interleaved per thread, threads per CTA).  A context uses one variant per
 * kernel; pyiid_gb300's autotuner times them on the caller's sizes and sets
 * the fastest.  No reference counterpart (the reference's numba launches are
 * fixed, atomics/gpu_atomics.py:120-184).
 *   kernel: PYIID_KERNEL_FQ (pyiid_fq and the F(Q) part of the batched call),
 *           PYIID_KERNEL_GRAD_FQ (pyiid_grad_fq), PYIID_KERNEL_FQ_GRAD
 *           (pyiid_fq_grad), PYIID_KERNEL_ADJOINT
 *           (the gradient of pyiid_batch_potential_grad: variant 0 evaluates
 *           each unordered pair once, variant 1 twice) or PYIID_KERNEL_MLP
 *           (the 32-128-128 surrogate network of pyiid_surrogate_forces:
 *           variant 0 register-resident mma.sync, params {16 atoms per warp,
 *           0, 256 threads}; variant 1 on tcgen05 tensor memory, params
 *           {128 atoms per CTA, 1, 128 threads}; variant 2 on tcgen05 with
 *           two 128-atom tiles in flight per CTA and two threads per row,
 *           params {256, 1, 512}; the default).
 *   params (pyiid_variant_info): {bins per thread, pairs per thread, threads
 *   per CTA}; pairs per thread <= 0 marks the packed (FP32x2) even/odd
 *   kernels (0: one pair per thread at a time, -2: two interleaved, -3/-4:
 *   the per-tile-pair group reduction at 3/4 CTAs per SM).  A new context
 *   starts on F(Q) variant 23 ({56, -3, 256}), MLP variant 2 and variant 0
 *   of the others. */
enum {
  PYIID_KERNEL_FQ = 0,
  PYIID_KERNEL_GRAD_FQ = 1,
  PYIID_KERNEL_ADJOINT = 2,
  PYIID_KERNEL_FQ_GRAD = 3,
  PYIID_KERNEL_MLP = 4
};
int pyiid_variant_count(int kernel);
int pyiid_variant_info(int kernel, int variant, int *params, int n_params);
int pyiid_set_variant(pyiid_ctx *ctx, int kernel, int variant);
int pyiid_get_variant(const pyiid_ctx *ctx, int kernel);

#ifdef __cplusplus
}
#endif

#endif /* PYIID_GB300_H */
