#!/usr/bin/env python
"""Exact F(Q) + full gradient evaluations per second on one GB300.

Workload (one "step" = one exact evaluation): a 20,000-atom spherical fcc Pt
particle (a = 3.92 A, the 20,000 sites nearest the origin, seeded N(0, 0.02^2)
displacements, float32), Q grid 0.5-30 1/A step 0.02 (1500 bins from Q = 0,
1475 returned), stand-in Pt form factor; outputs F(Q) [1475] and the full
gradient dF/dx [20000, 3, 1475] in the reference convention.  Inputs are
synthetic (seeded); the gradient output (354 MB) exceeds the 129 MB L2 and L2
is flushed between timed steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the reference's CPU path (the FP32 C port of its numba
code, oracle/debye_ref.c) on the host cores for the same workload, on a
bounded sample of pairs per step, and prints the same JSON line.
Under torchrun every rank evaluates its own copy (weak scaling, no
collective on the data path); rank 0 prints the line.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = 'exact F(Q)+grad evals/s'
N_ATOMS, A_PT, SIGMA, SEED = 20000, 3.92, 0.02, 2
QMIN, QMAX, QBIN = 0.5, 30.0, 0.02
FLOPS_GRAD_TERM = 20   # flop-equivalents per unordered pair-bin of dF/dx
FLOPS_F_TERM = 10      # ... of F(Q)
# FP32 lane operations the packed dF/dx inner loop issues per ordered
# pair-bin: per two bins 4 FFMA2/FADD2 of the recurrence and the derivative
# factor plus 3 FFMA2 of the x, y, z accumulation, plus 1 FADD2 of the bin
# factor (8 packed instructions = 16 lane operations per two bins).
LANE_OPS_GRAD_LOOP = 8
FP32_LANES_PER_SM = 128


def workload(n_atoms=None):
    from pyiid_gb300 import structures
    from pyiid_gb300.scatter_factors import species_tables
    n_atoms = n_atoms or N_ATOMS
    pos = structures.displaced(structures.fcc_nearest(A_PT, n_atoms), SIGMA,
                               SEED)
    n_bins = int(np.floor(QMAX / QBIN))
    k_begin = int(np.floor(QMIN / QBIN))
    sp, tab, _ = species_tables([78] * len(pos), QBIN, n_bins)
    return pos, sp, tab, n_bins, k_begin


def config_dict(n_bins, k_begin, n_atoms=N_ATOMS):
    """The workload block shared by both arms (identical dicts, so a reader
    can compare the GPU line with the reference line key by key); what
    differs between the arms (launch shapes, parallelism, the sampling of
    the CPU arm) goes in the line's ``arm`` block."""
    return {'workload': 'single fcc Pt nanoparticle, exact F(Q) + full dF/dx',
            'n_atoms': n_atoms, 'lattice_a': A_PT, 'sigma': SIGMA,
            'q_grid': f'{QMIN}-{QMAX} step {QBIN}',
            'bins_returned': n_bins - k_begin,
            'pairs': n_atoms * (n_atoms - 1) // 2,
            'l2': 'flushed between timed steps (256 MiB write)'}


def dist_env():
    rank = int(os.environ.get('RANK', '0'))
    world = int(os.environ.get('WORLD_SIZE', '1'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return rank, world, local


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ('clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
              'clocks_event_reasons.hw_slowdown,'
              'clocks_event_reasons.hw_thermal_slowdown,'
              'clocks_event_reasons.sw_thermal_slowdown,'
              'clocks_event_reasons.sw_power_cap')

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(),
                                 f'pyiid_gb300_clocks_{os.getpid()}.csv')

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, 'w')
            self.proc = subprocess.Popen(
                ['nvidia-smi', '-i', str(self.device),
                 f'--query-gpu={self.FIELDS}', '--format=csv,noheader,nounits',
                 '-lms', '200'], stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['unavailable']}
        rows = []
        for line in open(self.path):
            p = [x.strip() for x in line.split(',')]
            if len(p) < 8:
                continue
            try:
                rows.append((float(p[0]), float(p[1]), float(p[2]), p[4:8]))
            except ValueError:
                continue
        if not rows:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['no samples']}
        pw = np.array([r[2] for r in rows])
        load = [r for r in rows if r[2] >= 0.5 * pw.max()] or rows
        reasons = set()
        names = ('hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown',
                 'sw_power_cap')
        for r in load:
            for nm, v in zip(names, r[3]):
                if v.lower().startswith('active'):
                    reasons.add(nm)
        return {'sm_mhz': float(np.median([r[0] for r in load])),
                'sm_max_mhz': float(max(r[1] for r in rows)),
                'power_w_max': float(pw.max()),
                'samples': len(rows), 'reasons': sorted(reasons)}


# ------------------------------------------------------------- GPU arm
def fp32_peak_tflops(torch, dev):
    """Measured FP32 (CUDA-core) peak: cuBLAS SGEMM 8192^3, TF32 off."""
    torch.backends.cuda.matmul.allow_tf32 = False
    n = 8192
    a = torch.randn(n, n, device=dev)
    b = torch.randn(n, n, device=dev)
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(5):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        torch.matmul(a, b)
        e.record()
        e.synchronize()
        best = max(best, 2 * n ** 3 / (s.elapsed_time(e) * 1e-3) / 1e12)
    del a, b
    return best


def run_gpu(args, rank, world, local):
    import torch
    from pyiid_gb300 import debye
    from pyiid_gb300._native import context
    dev = torch.device('cuda', local)
    torch.cuda.set_device(dev)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl', device_id=dev)
        pg = dist
    pos, sp, tab, n_bins, k_begin = workload(args.n_atoms)
    n = len(pos)
    pairs = n * (n - 1) // 2
    k_ret = n_bins - k_begin
    pos_d = torch.as_tensor(pos, device=dev)
    fq = torch.empty(n_bins, dtype=torch.float32, device=dev)
    grad = torch.empty((n, 3, n_bins), dtype=torch.float32, device=dev)
    flush = torch.empty(256 * 2 ** 20 // 4, dtype=torch.float32, device=dev)
    ctx = context(local)

    def separate():
        debye.fq(pos_d, sp, tab, QBIN, k_begin, out=fq)
        debye.grad_fq(pos_d, sp, tab, QBIN, k_begin, out=grad)

    def fused():
        debye.fq_grad(pos_d, sp, tab, QBIN, k_begin, out_fq=fq, out_grad=grad)

    for _ in range(args.warmup):
        separate()
        fused()
    torch.cuda.synchronize()
    tuned = None
    step = fused
    if not args.no_tune:
        from pyiid_gb300 import autotune
        res = autotune.tune(pos_d, sp, tab, QBIN, k_begin, reps=2)
        res.update(autotune.tune_call(fused, kernels=('fq_grad',), reps=2))
        tuned = {k: dict(zip(('bins_per_thread', 'pairs_per_thread',
                              'threads'), autotune.variants(k)[v['best']][1]
                             .values())) for k, v in res.items()}
        # the faster of one pass (F and dF/dx together) and two passes
        step = min((fused, separate), key=lambda fn: time_ms(torch, fn, 3))
        torch.cuda.synchronize()
    one_pass = step is fused
    stream = torch.cuda.current_stream()
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)]
          for _ in range(args.steps)]
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    launches0 = ctx.launches
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for i in range(args.steps):
            flush.zero_()
            ev[i][0].record(stream)
            if one_pass:
                fused()
                ev[i][1].record(stream)
            else:
                debye.fq(pos_d, sp, tab, QBIN, k_begin, out=fq)
                ev[i][1].record(stream)
                debye.grad_fq(pos_d, sp, tab, QBIN, k_begin, out=grad)
            ev[i][2].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    launches = ctx.launches - launches0
    t_f = [ev[i][0].elapsed_time(ev[i][1]) for i in range(args.steps)]
    t_g = [ev[i][1].elapsed_time(ev[i][2]) for i in range(args.steps)]
    from pyiid_gb300.distributed import max_over_ranks
    ms_step = max_over_ranks(float(np.sum(t_f) + np.sum(t_g)) / args.steps,
                             device=dev)
    value = world / (ms_step * 1e-3)

    # end to end: pinned host positions -> device, F + dF/dx, results -> pinned host
    h_pos = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
    h_pos.copy_(torch.as_tensor(pos))
    h_fq = torch.empty(n_bins, dtype=torch.float32, pin_memory=True)
    h_grad = torch.empty((n, 3, n_bins), dtype=torch.float32, pin_memory=True)
    e2e_steps = max(3, min(args.steps, 10))

    def copy_out():
        # the step into device buffers, then explicit copies to pinned host
        pos_d.copy_(h_pos, non_blocking=True)
        step()
        h_fq.copy_(fq, non_blocking=True)
        h_grad.copy_(grad, non_blocking=True)

    def write_host():
        # one pass whose kernels write F and dF/dx straight into the pinned
        # host buffers over the host link, overlapped with the pair work
        pos_d.copy_(h_pos, non_blocking=True)
        debye.fq_grad(pos_d, sp, tab, QBIN, k_begin, out_fq=h_fq,
                      out_grad=h_grad)

    def e2e_time(fn):
        times = []
        for i in range(e2e_steps + 1):
            flush.zero_()
            s, e = (torch.cuda.Event(enable_timing=True),
                    torch.cuda.Event(enable_timing=True))
            s.record(stream)
            fn()
            e.record(stream)
            e.synchronize()
            if i:
                times.append(s.elapsed_time(e))
        return float(np.mean(times))

    e2e_copy_ms = e2e_time(copy_out)
    # correctness guard on what was timed: finite, nonzero
    assert torch.isfinite(grad).all() and fq[k_begin:].abs().sum() > 0
    h_grad.zero_()
    e2e_host_ms = e2e_time(write_host)
    # the host-written results are those of the same call on device buffers,
    # bit for bit
    fused()
    assert torch.equal(h_grad, grad.cpu()) and torch.equal(h_fq, fq.cpu())
    e2e_ms = max_over_ranks(min(e2e_copy_ms, e2e_host_ms), device=dev)
    e2e_path = ('kernels write the pinned host outputs (pyiid_fq_grad)'
                if e2e_host_ms < e2e_copy_ms else
                'device outputs, then cudaMemcpyAsync to pinned host')

    workloads = {}
    # the secondary workloads are single-GPU measurements: N = 1 only (with
    # N > 1 the other ranks would wait on rank 0 at the barrier below)
    if world == 1 and not args.no_workloads:
        for name, fn in (('fq_grad_au1000', run_fq_grad_au1000),
                         ('pdf_transforms_au1000', run_pdf_transforms),
                         ('batched_fq_256_alloys', run_batched),
                         ('hmc_64_chains_au1000', run_hmc),
                         ('delayed_acceptance_au1000', run_delayed_acceptance),
                         ('exact_incremental_mh', run_incremental_mh),
                         ('gcmc_au500', run_gcmc),
                         ('nuts_64_chains_au1000', run_nuts)):
            try:
                workloads[name] = fn(torch)
            except Exception as e:  # noqa: BLE001 -- reported, not fatal
                workloads[name] = {'error': f'{type(e).__name__}: {e}'}
    peak = fp32_peak_tflops(torch, dev) if rank == 0 else None
    if pg:
        pg.barrier()
        pg.destroy_process_group()
    if rank != 0:
        return None
    g_ms = float(np.mean(t_g))
    f_ms = float(np.mean(t_f))
    if one_pass:
        # the F and dF/dx of a step come from one launch: its time is t_f
        kernel = 'fqgrad2_kernel'
        k_ms = f_ms
        kernel_ms = {'fq_grad': f_ms}
        flops_term = FLOPS_GRAD_TERM + FLOPS_F_TERM
        # F(Q) adds 1 lane op per ordered pair-bin on the tiles J >= I
        lane_ops = LANE_OPS_GRAD_LOOP + 0.5
    else:
        kernel = ('gradfq2_kernel' if (tuned is None or
                                       tuned['grad_fq']['pairs_per_thread']
                                       <= 0) else 'gradfq_kernel')
        k_ms = g_ms
        kernel_ms = {'fq': f_ms, 'grad_fq': g_ms}
        flops_term = FLOPS_GRAD_TERM
        lane_ops = LANE_OPS_GRAD_LOOP
    achieved = pairs * k_ret * flops_term / (k_ms * 1e-3) / 1e12
    line = {
        'metric': METRIC, 'value': value, 'unit': 'evals/s', 'n_gpus': world,
        'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': ms_step,
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'fp32 (FP64 final reductions)', 'data': 'synthetic (seeded fcc Pt)',
        'config': config_dict(n_bins, k_begin, n),
        'arm': {'parallelism': f'replica x{world}',
                'launch_shapes': tuned or 'defaults',
                'path': ('one pass (pyiid_fq_grad)' if one_pass
                         else 'two passes (pyiid_fq, pyiid_grad_fq)')},
        'kernel_ms': kernel_ms,
        'pair_bin_terms_per_s': 2 * pairs * k_ret / (ms_step * 1e-3),
        'wall_s_timed_region': wall,
        'gpu_launches': int(launches),
        'e2e': {'value': world / (e2e_ms * 1e-3), 'unit': 'evals/s',
                'h2d_bytes_per_step': int(h_pos.numel() * 4),
                'd2h_bytes_per_step': int(h_fq.numel() * 4 + h_grad.numel() * 4),
                'path': e2e_path,
                'ms_copy_out': e2e_copy_ms, 'ms_kernels_write_host': e2e_host_ms},
        'roofline': {
            'bound': 'fp32',
            'kernel': kernel,
            'achieved': achieved, 'peak': peak, 'unit': 'TFLOP/s',
            'frac': achieved / peak if peak else None,
            'peak_source': 'measured live: cuBLAS SGEMM 8192^3 (TF32 off)',
            'algorithmic_flops_per_launch': pairs * k_ret * flops_term,
            'traffic': traffic_from_profile(kernel),
        },
        'clocks': clk.summary(),
    }
    line['roofline']['issue'] = issue_roofline(
        torch, dev, pairs, k_ret, k_ms, line['clocks'].get('sm_mhz'), kernel,
        lane_ops)
    # the same launch against HBM: its ncu DRAM bytes over its time
    hbm, traffic = measured_hbm_gbs(), line['roofline']['traffic']
    if hbm and traffic:
        gbs = traffic / (k_ms * 1e-3) / 1e9
        line['roofline']['hbm'] = {
            'achieved': gbs, 'peak': hbm, 'unit': 'GB/s', 'frac': gbs / hbm,
            'peak_source': 'MEASURED_PEAKS.json hbm_gbs (measured copy)'}
    if workloads:
        hmc, nuts = (workloads.get('hmc_64_chains_au1000'),
                     workloads.get('nuts_64_chains_au1000'))
        try:
            hmc_lf = hmc['hmc_iterations_per_s'] * 64 * 10
            nuts['batched']['hmc_leapfrog_steps_per_s'] = hmc_lf
            nuts['batched']['over_hmc_leapfrog_rate'] = (
                nuts['batched']['leapfrog_steps_per_s'] / hmc_lf)
        except (KeyError, TypeError):
            pass
        line['workloads'] = workloads
    return line


def run_gpu_sharded(args, rank, world, local):
    """The 20,000-atom particle split across the ranks (strong scaling):
    every rank evaluates its part of the tile list in one pass
    (pyiid_fq_grad_part: its atoms' complete gradient rows and the raw Debye
    sums of the pairs its tiles own), the K raw sums are all-reduced, and
    every rank forms F(Q) (pyiid_fq_from_sums).  A step is one evaluation of
    the one particle; the time is the maximum over ranks, including the
    all-reduce."""
    import torch
    from pyiid_gb300 import autotune, debye
    from pyiid_gb300._native import context
    from pyiid_gb300.distributed import max_over_ranks
    dev = torch.device('cuda', local)
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl', device_id=dev)
    pos, sp, tab, n_bins, k_begin = workload(args.n_atoms)
    n = len(pos)
    pairs = n * (n - 1) // 2
    k_ret = n_bins - k_begin
    pos_d = torch.as_tensor(pos, device=dev)
    grad = torch.zeros((n, 3, n_bins), dtype=torch.float32, device=dev)
    flush = torch.empty(256 * 2 ** 20 // 4, dtype=torch.float32, device=dev)
    ctx = context(local)
    out = {}

    def step():
        sums, _, rows = debye.fq_grad_part(pos_d, sp, tab, QBIN, k_begin,
                                           rank, world, out_grad=grad)
        if dist is not None:
            dist.all_reduce(sums, op=dist.ReduceOp.SUM)
        out['fq'] = debye.fq_from_sums(sp, tab, k_begin, sums)
        out['rows'] = rows

    for _ in range(args.warmup):
        step()
    if not args.no_tune:
        autotune.tune_call(step, kernels=('fq_grad',), reps=2)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    ev = [(torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = ctx.launches
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for s, e in ev:
            flush.zero_()
            s.record(stream)
            step()
            e.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    launches = ctx.launches - launches0
    ms_step = max_over_ranks(float(np.mean([s.elapsed_time(e) for s, e in ev])),
                             device=dev)
    own = torch.as_tensor(np.flatnonzero(out['rows']), device=dev)
    h_pos = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
    h_pos.copy_(torch.as_tensor(pos))
    h_fq = torch.empty(n_bins, dtype=torch.float32, pin_memory=True)
    h_rows = torch.empty((len(own), 3, n_bins), dtype=torch.float32,
                         pin_memory=True)
    times = []
    for i in range(max(3, min(args.steps, 10)) + 1):
        flush.zero_()
        s, e = (torch.cuda.Event(enable_timing=True),
                torch.cuda.Event(enable_timing=True))
        s.record(stream)
        pos_d.copy_(h_pos, non_blocking=True)
        step()
        h_fq.copy_(out['fq'], non_blocking=True)
        h_rows.copy_(grad.index_select(0, own), non_blocking=True)
        e.record(stream)
        e.synchronize()
        if i:
            times.append(s.elapsed_time(e))
    e2e_ms = max_over_ranks(float(np.mean(times)), device=dev)
    assert torch.isfinite(grad).all() and out['fq'][k_begin:].abs().sum() > 0
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    if rank != 0:
        return None
    return {
        'metric': METRIC, 'value': 1.0 / (ms_step * 1e-3), 'unit': 'evals/s',
        'n_gpus': world, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': ms_step, 'higher_is_better': True,
        'scaling': 'strong', 'vs_baseline': None,
        'dtype': 'fp32 (FP64 final reductions)',
        'data': 'synthetic (seeded fcc Pt)',
        'config': config_dict(n_bins, k_begin, n),
        'arm': {'parallelism': f'one particle split over {world} ranks '
                               '(tile ranges; all-reduce of the K raw sums)',
                'path': 'pyiid_fq_grad_part + pyiid_fq_from_sums'},
        'pair_bin_terms_per_s': 2 * pairs * k_ret / (ms_step * 1e-3),
        'wall_s_timed_region': wall,
        'gpu_launches': int(launches),
        'e2e': {'value': 1.0 / (e2e_ms * 1e-3), 'unit': 'evals/s',
                'h2d_bytes_per_step': int(h_pos.numel() * 4),
                'd2h_bytes_per_step': int(h_fq.numel() * 4 +
                                          h_rows.numel() * 4)},
        'clocks': clk.summary(),
    }


def issue_roofline(torch, dev, pairs, k_ret, k_ms, sm_mhz, kernel, lane_ops):
    """FP32 issue roofline of the dF/dx (or one-pass F + dF/dx) launch:
    lane operations its inner loop issues per second (each unordered
    pair-bin is evaluated for both atoms) over the SMs' FP32 lane capacity
    at the median SM clock sampled during the timed region.  Seeds and pair
    records are not counted."""
    if kernel not in ('gradfq2_kernel', 'fqgrad2_kernel') or not sm_mhz:
        return None
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    achieved = 2 * pairs * k_ret * lane_ops / (k_ms * 1e-3) / 1e12
    peak = sms * FP32_LANES_PER_SM * sm_mhz * 1e6 / 1e12
    return {'lane_ops_per_ordered_pair_bin': lane_ops,
            'achieved': achieved, 'peak': peak, 'unit': 'T lane-op/s',
            'frac': achieved / peak,
            'peak_source': f'{sms} SMs x {FP32_LANES_PER_SM} FP32 lanes x '
                           f'{sm_mhz:.0f} MHz (median sampled clock)',
            'counted': 'inner loop only (per-pair seeds and records excluded)'}


def time_ms(torch, fn, reps):
    """Mean CUDA-event time of fn() over reps calls after one warm call."""
    fn()
    s, e = (torch.cuda.Event(enable_timing=True),
            torch.cuda.Event(enable_timing=True))
    s.record()
    for _ in range(reps):
        fn()
    e.record()
    e.synchronize()
    return s.elapsed_time(e) / reps


def traffic_from_profile(kernel):
    """DRAM bytes per launch of the 20,000-atom workload's dominant kernel
    from its committed ncu summary, if any."""
    p = os.path.join(REPO, 'profiles', f'{kernel}_pt20000.md')
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith('dram_bytes_per_launch_full_size:'):
            try:
                return float(line.split(':', 1)[1].split()[0])
            except ValueError:
                return None
    return None


# ----------------------------------------------------- secondary workloads
def batched_workload():
    """256 fcc Au/Pt random alloys, N ~ U{55..2000} (seed 3), a = 4.0 A,
    sigma = 0.05 A, Q 0.1-25 1/A step 0.05."""
    from pyiid_gb300 import structures
    from pyiid_gb300.scatter_factors import species_tables
    sizes = np.random.default_rng(3).integers(55, 2001, 256)
    sites = structures.fcc_nearest(4.0, int(sizes.max()))
    pos, nums = [], []
    for b, n in enumerate(sizes):
        r = np.random.default_rng(3 + b)
        nums.append(np.where(r.random(n) < 0.5, 78, 79))
        pos.append((sites[:n] + r.normal(0, 0.05, (n, 3))).astype(np.float32))
    offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int32)
    sp, tab, _ = species_tables(np.concatenate(nums), 0.05, 500)
    return np.concatenate(pos), sp, offsets, tab, sizes


def run_batched(torch, steps=5):
    """Configuration 3: F(Q) of all 256 configurations per step, one graph
    replay (one pair-sum launch + one finishing launch), with the F(Q) launch
    shape tuned on this batch."""
    from pyiid_gb300 import autotune
    with autotune.variant_scope():
        return _run_batched(torch, steps)


def _run_batched(torch, steps):
    from pyiid_gb300 import autotune, debye
    from pyiid_gb300._native import context
    pos, sp, off, tab, sizes = batched_workload()
    p = torch.as_tensor(pos, device='cuda')
    out = torch.empty((len(sizes), 500), dtype=torch.float32, device='cuda')
    tuned = autotune.tune_call(
        lambda: debye.batch_fq(p, sp, off, tab, 0.05, 2, out=out),
        kernels=('fq',), reps=2)
    ctx = context()

    def graph_ms(variant, n=steps):
        """mean time of n replays of the batch captured in a CUDA graph"""
        ctx.set_variant('fq', variant)
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            for _ in range(3):
                debye.batch_fq(p, sp, off, tab, 0.05, 2, out=out)
        torch.cuda.current_stream().wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            debye.batch_fq(p, sp, off, tab, 0.05, 2, out=out)
        g.replay()
        torch.cuda.synchronize()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record()
        for _ in range(n):
            g.replay()
        ev1.record()
        ev1.synchronize()
        return ev0.elapsed_time(ev1) / n

    # the two launch forms of the group-reduction kernel, same bins per
    # thread: one CTA per work unit (hardware dispatch in largest-first
    # order) and the persistent form (resident CTAs, device work counter)
    shapes = {(i['bins_per_thread'], i['pairs_per_thread']): idx
              for idx, i in autotune.variants('fq')}
    forms = {}
    for L in (56, 48):
        forms[f'{L}_bins_per_thread'] = {
            'one_cta_per_unit_ms': graph_ms(shapes[(L, -3)], 10),
            'persistent_ms': graph_ms(shapes[(L, -13)], 10)}
    best = tuned['fq']['best']
    ms = graph_ms(best)
    info = dict(autotune.variants('fq'))[best]
    persistent = info['pairs_per_thread'] == -13
    pairs = int(np.sum(sizes.astype(np.int64) * (sizes - 1) // 2))
    assert torch.isfinite(out).all()
    # FP32 issue roofline: the F(Q) loop issues 3 lane-ops per unordered
    # pair-bin (per two bins: FFMA2 + FFMA2 recurrence, FADD2/FFMA2 sum)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    lane_peak = sms * FP32_LANES_PER_SM * 2.07e9 / 1e12
    lane = pairs * 498 * 3 / (ms * 1e-3) / 1e12
    return {'workload': '256 fcc Au/Pt alloys, N~U{55..2000}, Q 0.1-25 step 0.05',
            'atoms': int(sizes.sum()), 'pairs': pairs,
            'roofline': {'bound': 'fp32 issue', 'kernel': 'fq_pair3_kernel',
                         'achieved': lane, 'peak': lane_peak,
                         'unit': 'T lane-op/s', 'frac': lane / lane_peak,
                         'counted': '3 lane-ops per unordered pair-bin, '
                                    'whole batch (pair sums and finish)'},
            'ms_per_batch': ms, 'configs_per_s': len(sizes) / (ms * 1e-3),
            'pair_bin_terms_per_s': pairs * 498 / (ms * 1e-3),
            'fq_variant': best,
            'fq_shape': {'bins_per_thread': info['bins_per_thread'],
                         'persistent': persistent},
            'launch_forms': forms,
            'launch': ('CUDA graph replay: counter reset + 1 persistent '
                       'pair-sum + 1 finishing kernel') if persistent else
                      ('CUDA graph replay: 1 pair-sum (one CTA per work '
                       'unit) + 1 finishing kernel')}


def run_fq_grad_au1000(torch, reps=100, cpu_reps=2):
    """1,000-atom fcc Au (a = 4.08, sigma = 0.05, Q 0.1-25 step 0.05): exact
    F(Q) + full dF/dx of one configuration per evaluation, device-resident
    and end to end (host positions in, F and dF/dx back to pinned host), with
    the launch shapes tuned on this size; beside it full evaluations of the
    FP32 port of the reference CPU path on all host cores, same inputs."""
    from pyiid_gb300 import autotune
    with autotune.variant_scope():
        return _run_fq_grad_au1000(torch, reps, cpu_reps)


def _run_fq_grad_au1000(torch, reps, cpu_reps):
    from pyiid_gb300 import autotune, debye, structures
    from pyiid_gb300.scatter_factors import species_tables
    n, qbin = 1000, 0.05
    pos = structures.displaced(structures.fcc_nearest(4.08, n), 0.05, 4)
    n_bins, k_begin = 500, 2
    sp, tab, _ = species_tables([79] * n, qbin, n_bins)
    pos_d = torch.as_tensor(pos, device='cuda')
    fq = torch.empty(n_bins, dtype=torch.float32, device='cuda')
    grad = torch.empty((n, 3, n_bins), dtype=torch.float32, device='cuda')
    flush = torch.empty(256 * 2 ** 20 // 4, dtype=torch.float32, device='cuda')

    def separate():
        debye.fq(pos_d, sp, tab, qbin, k_begin, out=fq)
        debye.grad_fq(pos_d, sp, tab, qbin, k_begin, out=grad)

    def fused():
        debye.fq_grad(pos_d, sp, tab, qbin, k_begin, out_fq=fq, out_grad=grad)

    tuned = autotune.tune_call(separate, kernels=('fq', 'grad_fq'), reps=5)
    tuned.update(autotune.tune_call(fused, kernels=('fq_grad',), reps=5))
    evaluate = min((fused, separate), key=lambda fn: time_ms(torch, fn, 5))
    for _ in range(3):
        evaluate()
    stream = torch.cuda.current_stream()
    ev = [(torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    torch.cuda.synchronize()
    for s, e in ev:
        flush.zero_()
        s.record(stream)
        evaluate()
        e.record(stream)
    torch.cuda.synchronize()
    ms = float(np.mean([s.elapsed_time(e) for s, e in ev]))
    h_pos = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
    h_pos.copy_(torch.as_tensor(pos))
    h_fq = torch.empty(n_bins, dtype=torch.float32, pin_memory=True)
    h_grad = torch.empty((n, 3, n_bins), dtype=torch.float32, pin_memory=True)
    def copy_out():
        pos_d.copy_(h_pos, non_blocking=True)
        evaluate()
        h_fq.copy_(fq, non_blocking=True)
        h_grad.copy_(grad, non_blocking=True)

    def write_host():
        # the kernels write F and dF/dx straight into the pinned host buffers
        pos_d.copy_(h_pos, non_blocking=True)
        debye.fq_grad(pos_d, sp, tab, qbin, k_begin, out_fq=h_fq,
                      out_grad=h_grad)

    def e2e_time(fn):
        e2e = []
        for i in range(reps + 1):
            flush.zero_()
            s, e = (torch.cuda.Event(enable_timing=True),
                    torch.cuda.Event(enable_timing=True))
            s.record(stream)
            fn()
            e.record(stream)
            e.synchronize()
            if i:
                e2e.append(s.elapsed_time(e))
        return float(np.mean(e2e))

    e2e_copy_ms = e2e_time(copy_out)
    assert torch.isfinite(grad).all() and fq[k_begin:].abs().sum() > 0
    h_grad.zero_()
    e2e_host_ms = e2e_time(write_host)
    fused()
    assert torch.equal(h_grad, grad.cpu()) and torch.equal(h_fq, fq.cpu())
    e2e_ms = min(e2e_copy_ms, e2e_host_ms)

    from oracle import build_oracle, debye_c
    build_oracle.build()
    per_atom = tab[sp]
    pairs = n * (n - 1) // 2
    debye_c.port_tasks(pos, per_atom, qbin, 2048, pairs, True, True)
    t = []
    for _ in range(cpu_reps):
        t0 = time.perf_counter()
        _, _, used = debye_c.port_tasks(pos, per_atom, qbin, 2048, pairs,
                                        True, True)
        t.append(time.perf_counter() - t0)
    cpu = 1.0 / float(np.mean(t))
    gpu = 1e3 / ms
    single = single_config_au1000(torch)
    # the one-pass kernel's FP32 issue roofline at this size: lane operations
    # of its inner loop (8.5 per ordered pair-bin) over 152 SMs x 128 lanes
    # at the maximum SM clock, with the whole call's time (kernel, part
    # combine and finish)
    k_ret = n_bins - k_begin
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    lane_peak = sms * FP32_LANES_PER_SM * 2.07e9 / 1e12
    lane = 2 * pairs * k_ret * (LANE_OPS_GRAD_LOOP + 0.5) / (ms * 1e-3) / 1e12
    roof = {'bound': 'fp32 issue', 'kernel': 'fqgrad2_kernel',
            'achieved': lane, 'peak': lane_peak, 'unit': 'T lane-op/s',
            'frac': lane / lane_peak,
            'peak_source': f'{sms} SMs x {FP32_LANES_PER_SM} lanes x 2070 MHz',
            'flop_eq_tflops': pairs * k_ret * (FLOPS_GRAD_TERM +
                                               FLOPS_F_TERM) / (ms * 1e-3) / 1e12}
    return {'workload': '1000-atom fcc Au, exact F(Q) + full dF/dx, '
                        'Q 0.1-25 step 0.05 (498 bins returned)',
            'pairs': pairs, 'ms_per_eval': ms, 'evals_per_s': gpu,
            'e2e_evals_per_s': 1e3 / e2e_ms,
            'e2e_bytes': {'h2d': int(h_pos.numel() * 4),
                          'd2h': int((h_fq.numel() + h_grad.numel()) * 4)},
            'e2e_ms': {'copy_out': e2e_copy_ms,
                       'kernels_write_host': e2e_host_ms},
            'variants': {k: v['best'] for k, v in tuned.items()},
            'path': ('one pass (pyiid_fq_grad)' if evaluate is fused
                     else 'two passes (pyiid_fq, pyiid_grad_fq)'),
            'l2': 'flushed between timed evaluations (256 MiB write)',
            'cpu_port': {'evals_per_s': cpu, 'cores': int(used),
                         'sample': f'{cpu_reps} full evaluations (all pairs, '
                                   f'F and dF/dx, {n_bins} bins) after one '
                                   'warm-up'},
            'gpu_over_cpu_port': gpu / cpu,
            'e2e_over_cpu_port': 1e3 / e2e_ms / cpu,
            'roofline': roof,
            'single_configuration': single}


def single_config_au1000(torch, reps=50):
    """One 1,000-atom Au configuration through the calls a drop-in Calc1D
    or ElasticScatter user makes per step: the exact Rw and its gradient on
    the PDF grid (pyiid_batch_potential_grad, one configuration) and F(Q)
    on Q 0.1-25 step 0.05 (pyiid_fq)."""
    from pyiid_gb300 import debye, structures
    from pyiid_gb300.sampling import PDFPotential, experiment_grids
    from pyiid_gb300.scatter_factors import species_tables
    exp, qb, nb, rg = experiment_grids(None)
    ref = structures.fcc_nearest(4.08, 1000).astype(np.float32)
    sp, tab, _ = species_tables([79] * 1000, qb, nb)
    f = debye.fq(ref, sp, tab, qb)
    gobs = debye.pdf(f, qb, exp['rstep'], rg, exp['qmin']).cpu().numpy()
    pot = PDFPotential([79] * 1000, gobs, None, conv=100.0, n_configs=1)
    x = torch.as_tensor(structures.displaced(ref, 0.05, 4), device='cuda')
    sp2, tab2, _ = species_tables([79] * 1000, 0.05, 500)
    fo = torch.empty(500, device='cuda')
    return {'potential_and_gradient_ms':
                time_ms(torch, lambda: pot.evaluate(x), reps),
            'fq_ms': time_ms(torch, lambda: debye.fq(x, sp2, tab2, 0.05, 2,
                                                     out=fo), reps),
            'fq_noalloc_ms': time_ms(torch, lambda: fq_noalloc(
                x, sp2, tab2, 0.05, 2, fo), reps)}


def fq_noalloc(pos_t, sp, tab, qbin, kb, out):
    """One pyiid_fq_noalloc call through the C ABI (it synchronizes)."""
    import ctypes
    import torch
    from pyiid_gb300 import _native
    ctx = _native.context(pos_t.device.index)
    sp = np.ascontiguousarray(sp, np.int32)
    tab = np.ascontiguousarray(tab, np.float32)
    ctx.call('pyiid_fq_noalloc', ctypes.c_void_p(pos_t.data_ptr()),
             sp.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), len(sp),
             tab.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), tab.shape[0],
             tab.shape[1], float(qbin), int(kb), ctypes.c_void_p(out.data_ptr()))
    return out


def measured_peak(key):
    """A peak measured on this part (MEASURED_PEAKS.json: hbm_gbs,
    bf16_tflops, ...), or None."""
    try:
        with open(os.path.join(REPO, 'MEASURED_PEAKS.json')) as f:
            return float(json.load(f)[key])
    except (OSError, ValueError, KeyError):
        return None


def measured_hbm_gbs():
    """HBM copy bandwidth measured on this part (MEASURED_PEAKS.json)."""
    return measured_peak('hbm_gbs')


def run_pdf_transforms(torch, reps=50):
    """The F(Q) -> G(r) transforms on the 1,000-atom Au grids (Q_pdf step
    0.0756865, 330 bins; r 0-40 step 0.01, 4000 points):
      forward: G(r) of 64 configurations per call (pyiid_pdf); algorithmic
               bytes per configuration 4 K' R (T) + 4 K' + 8 R;
      grad_pdf: the compat [N, 3, K'] -> [N, 3, R] map at N = 1000
               (pyiid_grad_pdf): 2 (3N) K' R flops, 4 (3N) K' + 8 (3N) R
               bytes (+ T).
    Device-resident inputs, CUDA events, mean over reps calls."""
    from pyiid_gb300 import debye
    from pyiid_gb300.sampling import experiment_grids
    exp, qb, nb, rg = experiment_grids(None)
    n_r, b, n = len(rg), 64, 1000
    g = torch.Generator(device='cuda').manual_seed(7)
    fq = torch.randn((b, nb), device='cuda', generator=g)
    gfq = torch.randn((n, 3, nb), device='cuda', generator=g)

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        s, e = (torch.cuda.Event(enable_timing=True),
                torch.cuda.Event(enable_timing=True))
        s.record()
        for _ in range(reps):
            fn()
        e.record()
        e.synchronize()
        return s.elapsed_time(e) / reps

    fwd = lambda: debye.pdf(fq, qb, exp['rstep'], rg, exp['qmin'])  # noqa: E731
    bwd = lambda: debye.grad_pdf(gfq, qb, exp['rstep'], rg, exp['qmin'])  # noqa: E731
    ms_f = timed(fwd)
    ms_g = timed(bwd)
    assert torch.isfinite(fwd()).all() and torch.isfinite(bwd()).all()
    hbm = measured_hbm_gbs()
    fwd_bytes = b * (4 * nb * n_r + 4 * nb + 8 * n_r)
    g_flops = 2 * 3 * n * nb * n_r
    g_bytes = 4 * 3 * n * nb + 8 * 3 * n * n_r + 4 * nb * n_r
    peak = fp32_peak_tflops(torch, torch.device('cuda'))
    bf16 = measured_peak('bf16_tflops')
    fwd_gbs = fwd_bytes / (ms_f * 1e-3) / 1e9
    return {
        'workload': 'G(r) transforms, 1000-atom Au grids (K\' 330, R 4000)',
        'forward': {'configs': b, 'ms': ms_f,
                    'algorithmic_bytes': fwd_bytes,
                    'achieved_gbs': fwd_gbs,
                    'hbm_peak_gbs': hbm,
                    'note': 'T (5.3 MB) is read from L2 after the first '
                            'configuration of a call, so the algorithmic '
                            'rate can exceed the HBM copy rate'},
        'grad_pdf': {'n_atoms': n, 'ms': ms_g, 'flops': g_flops,
                     'achieved_tflops': g_flops / (ms_g * 1e-3) / 1e12,
                     'fp32_peak_tflops': peak,
                     'frac': g_flops / (ms_g * 1e-3) / 1e12 / peak,
                     'frac_of': 'live FP32 SGEMM (the accuracy the result '
                                'keeps)',
                     # three FP16 products per multiply-add on tcgen05
                     'tensor': {
                         'achieved_tflops': 3 * g_flops / (ms_g * 1e-3)
                         / 1e12,
                         'peak_tflops': bf16,
                         'frac': (3 * g_flops / (ms_g * 1e-3) / 1e12 / bf16
                                  if bf16 else None),
                         'peak_source': 'MEASURED_PEAKS.json bf16_tflops '
                                        '(cuBLAS bf16, burst)'},
                     'algorithmic_bytes': g_bytes,
                     'achieved_gbs': g_bytes / (ms_g * 1e-3) / 1e9,
                     'hbm_peak_gbs': hbm,
                     'hbm_frac': (g_bytes / (ms_g * 1e-3) / 1e9 / hbm
                                  if hbm else None)},
    }


def run_hmc(torch, iters=6):
    """Configuration 4: 1,000-atom fcc Au, 64 chains, 10 leapfrog steps,
    dt = 1e-3, T = 300 K, E = 100 * Rw against the undisplaced G(r); one
    CUDA-graph replay per HMC iteration of all chains, with the F(Q) and
    adjoint launch shapes tuned on the batched evaluation."""
    from pyiid_gb300 import autotune
    with autotune.variant_scope():
        return _run_hmc(torch, iters)


def _run_hmc(torch, iters):
    from pyiid_gb300 import autotune, structures
    from pyiid_gb300.sampling import PDFPotential, BatchedHMC, experiment_grids
    from pyiid_gb300.scatter_factors import species_tables
    from pyiid_gb300 import debye
    exp, qb, nb, rg = experiment_grids(None)
    ref = structures.fcc_nearest(4.08, 1000).astype(np.float32)
    sp, tab, _ = species_tables([79] * 1000, qb, nb)
    f = debye.fq(ref, sp, tab, qb)
    gobs = debye.pdf(f, qb, exp['rstep'], rg, exp['qmin']).cpu().numpy()
    pot = PDFPotential([79] * 1000, gobs, None, conv=100.0, n_configs=64)
    xs = np.stack([structures.displaced(ref, 0.05, 4 + c) for c in range(64)])
    x0 = torch.as_tensor(xs.reshape(-1, 3).astype(np.float32), device='cuda')
    tuned = autotune.tune_call(lambda: pot.evaluate(x0), reps=2)
    hmc = BatchedHMC(pot, xs, temperature=300.0, dt=1e-3, n_steps=10, seed=4,
                     graph=True)
    hmc.step(2)
    torch.cuda.synchronize()
    hmc.accepted.zero_()
    hmc.proposed = 0
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    hmc.step(iters)
    ev1.record()
    ev1.synchronize()
    s = ev0.elapsed_time(ev1) * 1e-3
    acc = int(hmc.accepted.sum().item())
    # one force evaluation of all 64 chains, for reference
    x = hmc.positions()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    pot.evaluate(x)
    e0.record()
    for _ in range(3):
        pot.evaluate(x)
    e1.record()
    e1.synchronize()
    ev_ms = e0.elapsed_time(e1) / 3
    # one evaluation = F(Q) of the 64 configurations (3 lane-ops per unordered
    # pair-bin) + the symmetric adjoint (5 lane-ops per unordered pair-bin)
    # on the PDF grid
    k_pdf = pot.n_bins
    pairs64 = 64 * 1000 * 999 // 2
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    lane_peak = sms * FP32_LANES_PER_SM * 2.07e9 / 1e12
    lane = pairs64 * k_pdf * (3 + 5) / (ev_ms * 1e-3) / 1e12
    return {'workload': '1000-atom fcc Au, 64 chains, 10 leapfrog x dt 1e-3, 300 K, E = 100 Rw',
            'roofline': {'bound': 'fp32 issue',
                         'kernel': 'fq_pair3_kernel + adjoint_sym_kernel',
                         'achieved': lane, 'peak': lane_peak,
                         'unit': 'T lane-op/s', 'frac': lane / lane_peak,
                         'counted': '3 (F) + 5 (adjoint) lane-ops per '
                                    'unordered pair-bin, whole evaluation'},
            'hmc_iterations_per_s': iters / s,
            'accepted_steps_per_s': acc / s,
            'acceptance': acc / (iters * 64),
            'ms_per_iteration': 1e3 * s / iters,
            'ms_per_force_eval_64_chains': ev_ms,
            'variants': {k: v['best'] for k, v in tuned.items()},
            'launch': 'CUDA graph replay per HMC iteration (11 batched exact evaluations)'}


def ess_sum(traces):
    """Summed effective sample size of per-chain traces [T, B]: Geyer's
    initial positive sequence on each chain's autocorrelation (pairs of
    lags summed until a pair turns negative)."""
    x = np.asarray(traces, np.float64)
    T, B = x.shape
    total = 0.0
    for c in range(B):
        y = x[:, c] - x[:, c].mean()
        v = float(y @ y) / T
        if v <= 0:
            continue
        ac = np.array([float(y[:T - k] @ y[k:]) / T / v for k in range(T)])
        s = 0.0
        for k in range(1, T - 1, 2):
            pair = ac[k] + ac[k + 1]
            if pair < 0:
                break
            s += pair
        total += T / (1.0 + 2.0 * s)
    return total


def run_delayed_acceptance(torch, iters=30, pool=256, pretrain_steps=300):
    """Configuration 5, delayed-acceptance HMC (surrogate-driven 10-step
    trajectories, two-stage acceptance with the exact Debye potential)
    against plain exact batched HMC, both on the 64 chains of the 1,000-atom
    Au particle (dt = 1e-3, 300 K, E = 100 Rw).  The surrogate (RBF 32
    centres / 8 A -> MLP 32-128-128-1, BF16) is pre-trained on exact Rw of
    ``pool`` displaced particles (sigma 0.01-0.2 A) and then trained online
    every 10 iterations on the exact evaluations of its own second stage;
    the same run with the untrained network shows what the training gains.
    Accepted steps/s and ESS(Rw)/s (Geyer's initial positive sequence over
    the iterations of every chain) for each sampler; the pre-training time is
    reported, not amortised."""
    from pyiid_gb300 import structures
    from pyiid_gb300.sampling import BatchedHMC, PDFPotential
    from pyiid_gb300.surrogate import RBFMLPSurrogate, DelayedAcceptanceHMC
    pot, start = setup_au1000_chains(torch)
    gobs = pot.gobs.cpu().numpy()
    ref = structures.fcc_nearest(4.08, 1000).astype(np.float32)
    t0 = time.perf_counter()
    sig = np.random.default_rng(5).uniform(0.01, 0.2, pool)
    xs = np.stack([structures.displaced(ref, s, 5000 + i)
                   for i, s in enumerate(sig)])
    ppot = PDFPotential([79] * 1000, gobs, None, n_configs=pool)
    rw = ppot.evaluate(torch.as_tensor(xs.reshape(-1, 3), device='cuda'),
                       want_grad=False)[0].clone()
    trained = RBFMLPSurrogate(seed=0, lr=3e-3)
    fb = trained.features(xs.reshape(-1, 3), ppot.offsets)
    for _ in range(pretrain_steps):
        loss = trained.train_step(fb, ppot.offsets, rw)
    torch.cuda.synchronize()
    out = {'workload': '1000-atom fcc Au, 64 chains, 10 leapfrog x dt 1e-3, '
                       '300 K, E = 100 Rw; surrogate RBF(32, 8 A) -> MLP '
                       '32-128-128-1 BF16',
           'pretrain': {'seconds': time.perf_counter() - t0,
                        'configurations': pool, 'adam_steps': pretrain_steps,
                        'final_mse_rw': loss}}

    def timed(sampler, train_every=0):
        rws, ms = [], 0.0
        e0, e1 = (torch.cuda.Event(enable_timing=True) for _ in range(2))
        for i in range(iters):
            e0.record()
            sampler.step(1)
            e1.record()
            e1.synchronize()
            ms += e0.elapsed_time(e1)
            e = sampler.E if hasattr(sampler, 'E') else sampler.u
            rws.append((e / pot.conv).cpu().numpy())
            if train_every and (i + 1) % train_every == 0:
                t = time.perf_counter()
                sampler.train(steps=1, batch=16)
                torch.cuda.synchronize()
                ms += 1e3 * (time.perf_counter() - t)
        return ms * 1e-3, np.array(rws)

    hmc = BatchedHMC(pot, start, temperature=300.0, dt=1e-3, n_steps=10,
                     seed=4, graph=True)
    hmc.step(2)
    hmc.accepted.zero_()
    hmc.proposed = 0
    s, tr = timed(hmc)
    acc = int(hmc.accepted.sum().item())
    out['plain_hmc'] = {'accepted_steps_per_s': acc / s,
                        'acceptance': acc / (iters * 64),
                        'ms_per_iteration': 1e3 * s / iters,
                        'ess_rw_per_s': ess_sum(tr) / s,
                        'exact_evaluations_per_iteration': '10 with gradient'}
    for name, sur, every in (('delayed_acceptance', trained, 10),
                             ('delayed_acceptance_untrained',
                              RBFMLPSurrogate(seed=0), 0)):
        da = DelayedAcceptanceHMC(pot, sur, start, temperature=300.0,
                                  dt=1e-3, n_steps=10, seed=4, graph=True)
        da.step(2)
        da._reset_counters()
        s, tr = timed(da, every)
        a = da.acceptance()
        acc = int(da.accepted.sum().item())
        out[name] = {'accepted_steps_per_s': acc / s,
                     'acceptance': acc / (iters * 64),
                     'stage1_acceptance': float(a['stage1'].mean()),
                     'ms_per_iteration': 1e3 * s / iters,
                     'ess_rw_per_s': ess_sum(tr) / s,
                     'rms_stage2_log_ratio_kT': float(
                         (da.sum_dhs_err / (iters * 64)).sqrt()) / da.kT,
                     'online_training': (f'1 Adam step on 16 buffered '
                                         f'pairs every {every} iterations '
                                         '(timed)') if every
                     else 'none',
                     'exact_evaluations_per_iteration': '1 energy only',
                     'lists': da.check()}
    hp = out['plain_hmc']
    for name in ('delayed_acceptance', 'delayed_acceptance_untrained'):
        out[name]['over_plain_hmc_accepted'] = (
            out[name]['accepted_steps_per_s'] / hp['accepted_steps_per_s'])
        out[name]['over_plain_hmc_ess'] = (
            out[name]['ess_rw_per_s'] / max(hp['ess_rw_per_s'], 1e-300))
    return out


def run_delayed_acceptance_single_atom(torch, iters=20):
    """Single-atom delayed-acceptance Metropolis (sigma 0.1 A moves, the
    surrogate over every atom per proposal) against exact single-atom
    Metropolis by full re-evaluation and the O(N K) incremental sampler."""
    from pyiid_gb300 import structures, debye
    from pyiid_gb300.sampling import PDFPotential, experiment_grids
    from pyiid_gb300.scatter_factors import species_tables
    from pyiid_gb300.surrogate import (RBFMLPSurrogate, DelayedAcceptanceMH,
                                       ExactSingleAtomMH)
    exp, qb, nb, rg = experiment_grids(None)
    ref = structures.fcc_nearest(4.08, 1000).astype(np.float32)
    sp, tab, _ = species_tables([79] * 1000, qb, nb)
    gobs = debye.pdf(debye.fq(ref, sp, tab, qb), qb, exp['rstep'], rg,
                     exp['qmin']).cpu().numpy()
    sig = np.random.default_rng(5).uniform(0.01, 0.2, 256)
    pool = np.stack([structures.displaced(ref, s, 5000 + i)
                     for i, s in enumerate(sig)])
    ppot = PDFPotential([79] * 1000, gobs, None, n_configs=256)
    rw = ppot.evaluate(torch.as_tensor(pool.reshape(-1, 3), device='cuda'),
                       want_grad=False)[0].clone()
    sur = RBFMLPSurrogate(seed=0, lr=3e-3)
    fb = sur.features(pool.reshape(-1, 3), ppot.offsets)
    for _ in range(200):
        sur.train_step(fb, ppot.offsets, rw)
    start = np.stack([structures.displaced(ref, 0.05, 4 + c)
                      for c in range(64)])
    pot = PDFPotential([79] * 1000, gobs, None, conv=100.0, n_configs=64)
    out = {}
    for name, mk in (
            ('delayed_acceptance', lambda: DelayedAcceptanceMH(
                pot, sur, start, temperature=300, step=0.1, seed=6,
                train_every=5, train_steps=1, train_batch=32)),
            ('exact_single_atom_mh', lambda: ExactSingleAtomMH(
                pot, start, temperature=300, step=0.1, seed=6))):
        ch = mk()
        for _ in range(3):
            ch.iterate()
        torch.cuda.synchronize()
        a0, e0, p0 = ch.accepted, ch.exact_evals, ch.proposed
        t = time.perf_counter()
        for _ in range(iters):
            ch.iterate()
        torch.cuda.synchronize()
        dt = time.perf_counter() - t
        acc = ch.accepted - a0
        out[name] = {'accepted_steps_per_s': acc / dt,
                     'acceptance': acc / max(ch.proposed - p0, 1),
                     'exact_evals_per_accepted':
                         (ch.exact_evals - e0) / max(acc, 1)}
    out['exact_incremental_mh'] = run_incremental_mh(torch, pot, start)
    return out


def run_surrogate_forces(torch, reps=20):
    """The surrogate's energy and forces for the 64 x 1,000-atom chains of
    the delayed-acceptance workload (one pyiid_surrogate_forces call:
    neighbour-list descriptors, fused MLP forward and descriptor gradient,
    forces), after one neighbour-list build; mean CUDA-event time."""
    from pyiid_gb300.surrogate import RBFMLPSurrogate, DelayedAcceptanceHMC
    pot, start = setup_au1000_chains(torch)
    da = DelayedAcceptanceHMC(pot, RBFMLPSurrogate(seed=0), start,
                              temperature=300.0, dt=1e-3, n_steps=10, seed=4)
    x = da.x.clone()
    da._neighbours(x)
    ms = time_ms(torch, lambda: da.surrogate(x), reps)
    return {'workload': 'surrogate energy + forces, 64 x 1000-atom Au, '
                        '32 centres / 8 A, MLP 32-128-128-1',
            'ms_per_call': ms, 'atoms': int(x.shape[0]),
            'neighbour_list_ms': time_ms(torch, lambda: da._neighbours(x),
                                         reps),
            'max_neighbours': int(da.cnt.max().item())}


def setup_au1000_chains(torch, n_chains=64):
    """The 64-chain single-atom workload: 1,000-atom fcc Au (a = 4.08 A),
    gobs = G(r) of the undisplaced particle, chains started from seeded
    0.05 A displacements, E = 100 Rw on the default PDF grid."""
    from pyiid_gb300 import structures, debye
    from pyiid_gb300.sampling import PDFPotential, experiment_grids
    from pyiid_gb300.scatter_factors import species_tables
    exp, qb, nb, rg = experiment_grids(None)
    ref = structures.fcc_nearest(4.08, 1000).astype(np.float32)
    sp, tab, _ = species_tables([79] * 1000, qb, nb)
    gobs = debye.pdf(debye.fq(ref, sp, tab, qb), qb, exp['rstep'], rg,
                     exp['qmin']).cpu().numpy()
    start = np.stack([structures.displaced(ref, 0.05, 4 + c)
                      for c in range(n_chains)])
    pot = PDFPotential([79] * 1000, gobs, None, conv=100.0,
                       n_configs=n_chains)
    return pot, start


def run_incremental_mh(torch, pot=None, start=None, n_steps=8192):
    """Exact single-atom Metropolis with O(N K) energy changes
    (pyiid_mh_steps), 64 proposals per chain per CUDA-graph replay, a full
    re-synchronisation every 4096 steps included in the timing."""
    from pyiid_gb300.sampling import SingleAtomMC
    if pot is None:
        pot, start = setup_au1000_chains(torch)
    mc = SingleAtomMC(pot, start.reshape(-1, 3), temperature=300, sigma=0.1,
                      seed=6, graph=True, steps_per_replay=64)
    mc.step(256)
    torch.cuda.synchronize()
    a0 = int(mc.state['accepted'].sum().item())
    ev0, ev1 = (torch.cuda.Event(enable_timing=True) for _ in range(2))
    t = time.perf_counter()
    ev0.record()
    mc.step(n_steps)
    ev1.record()
    torch.cuda.synchronize()
    dt = time.perf_counter() - t
    acc = int(mc.state['accepted'].sum().item()) - a0
    props = n_steps * pot.n_configs
    # move_delta_kernel's loop: per two bins of one partner, 4 FFMA2 of the
    # two recurrences (old and new position) and 2-3 for their difference:
    # 3.25 lane-ops per pair term (one position, one bin)
    dev_s = ev0.elapsed_time(ev1) * 1e-3
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    lane_peak = sms * FP32_LANES_PER_SM * 2.07e9 / 1e12
    terms = props * 2 * 999 * pot.n_bins
    lane = terms * 3.25 / dev_s / 1e12
    return {'roofline': {'bound': 'latency (fp32 issue counted)',
                         'kernel': 'move_delta_kernel + move_gram_kernel',
                         'achieved': lane, 'peak': lane_peak,
                         'unit': 'T lane-op/s', 'frac': lane / lane_peak,
                         'counted': '3.25 lane-ops per pair term, whole '
                                    'step (two dependent launches of about '
                                    '42 M pair terms for 64 chains)'},
            'accepted_steps_per_s': acc / dt,
            'proposals_per_s': props / dt,
            'acceptance': acc / props,
            'us_per_step_all_chains': 1e6 * dt / n_steps,
            'device_us_per_step': 1e3 * ev0.elapsed_time(ev1) / n_steps,
            'exact_evals_per_accepted': props / max(acc, 1),
            'pair_terms_per_proposal': 2 * 999 * pot.n_bins}


# ------------------------------------------------------------- CPU arm
def cpu_sample(target_s=15.0, threads=0, n_atoms=None):
    """Time the FP32 reference-path port on a bounded sample of the workload's
    pairs (F and dF/dx tasks) and extrapolate to all pairs:
      t(eval) = t_fixed + P * (t(2 rounds) - t(1 round)) / (pairs per round)
    where t_fixed (per-thread [n,3,K] buffers and their one final sum) is
    the 1-round time minus its marginal part; a full evaluation pays it once.
    The returned value is therefore EXTRAPOLATED (``extrapolated`` True,
    ``pairs_timed`` of ``pairs_per_evaluation``)."""
    from oracle import debye_c
    pos, sp, tab, n_bins, k_begin = workload(n_atoms)
    per_atom = tab[sp]
    n = len(pos)
    pairs = n * (n - 1) // 2
    chunk = 2048
    nthreads = threads or os.cpu_count()

    def run(rounds):
        t0 = time.perf_counter()
        _, _, used = debye_c.port_tasks(pos, per_atom, QBIN, chunk,
                                        chunk * nthreads * rounds, True, True,
                                        nthreads)
        return time.perf_counter() - t0, used

    t1, used = run(1)
    rounds = max(2, int(target_s / max(t1, 1e-3)))
    t2, _ = run(rounds)
    per_pair = (t2 - t1) / (chunk * nthreads * (rounds - 1))
    fixed = max(0.0, t1 - per_pair * chunk * nthreads)
    t_eval = fixed + per_pair * pairs
    timed = chunk * nthreads * (rounds + 1)
    return {'value': 1.0 / t_eval, 'unit': 'evals/s', 'cores': int(used),
            'kind': 'port',
            'extrapolated': True,
            'pairs_timed': timed, 'pairs_per_evaluation': pairs,
            'sample': (f'{timed} of {pairs} pairs (all {n_bins} bins, F and '
                       f'dF/dx tasks of {chunk} pairs) timed in '
                       f'{t1 + t2:.1f} s; marginal {per_pair * 1e6:.2f} us/pair '
                       f'+ fixed {fixed:.2f} s, extrapolated to all pairs'),
            'seconds': t1 + t2}


def cpu_full_evaluations(sizes=(1000, 2000), threads=0):
    """Complete evaluations of the FP32 reference-path port (every pair,
    F(Q) and dF/dx, all bins of the workload's Q grid) on the first N sites
    of the same particle, timed without extrapolation; each also scaled by
    pairs to the workload's size for comparison with the sampled estimate."""
    from oracle import debye_c
    out = {}
    for n in sizes:
        pos, sp, tab, n_bins, k_begin = workload(n)
        pairs = n * (n - 1) // 2
        t0 = time.perf_counter()
        _, _, used = debye_c.port_tasks(pos, tab[sp], QBIN, 2048, pairs, True,
                                        True, threads)
        dt = time.perf_counter() - t0
        full = N_ATOMS * (N_ATOMS - 1) // 2
        out[f'n{n}'] = {'n_atoms': n, 'pairs': pairs, 'bins': n_bins,
                        'seconds_per_eval': dt, 'evals_per_s': 1.0 / dt,
                        'cores': int(used), 'extrapolated': False,
                        'scaled_by_pairs_to_workload_evals_per_s':
                            pairs / (dt * full)}
    return out


def run_reference(args, rank, world):
    if rank != 0:
        return None
    from oracle import build_oracle
    build_oracle.build()
    pos, sp, tab, n_bins, k_begin = workload()
    vals = []
    per_step = max(3.0, min(20.0, 60.0 / max(1, args.steps)))
    for i in range(args.warmup):
        cpu_sample(target_s=1.0)
    for i in range(args.steps):
        vals.append(cpu_sample(target_s=per_step))
    v = float(np.mean([x['value'] for x in vals]))
    base = dict(vals[-1])
    base['value'] = v
    full = cpu_full_evaluations() if getattr(args, 'full_cpu', True) else {}
    step_s = float(np.mean([x['seconds'] for x in vals]))
    return {
        'metric': METRIC, 'value': v, 'unit': 'evals/s', 'n_gpus': world,
        'steps': args.steps, 'warmup': args.warmup,
        # a step is one bounded sample of the workload's pairs: its measured
        # wall time; the value is the full evaluation rate extrapolated
        # from the samples
        'ms_per_step': 1e3 * step_s, 'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None, 'dtype': 'fp32 (FP64 sums)',
        'data': 'synthetic (seeded fcc Pt)', 'impl': 'reference',
        'config': config_dict(n_bins, k_begin),
        'arm': {'parallelism': 'host cores (OpenMP threads)',
                'path': 'FP32 loop-for-loop port of the reference numba CPU '
                        'path (cpu_flat.py + flat_multi_cpu_wrap.py)'},
        'extrapolated': True,
        'timed': {'pairs_per_step': int(np.mean([x['pairs_timed']
                                                 for x in vals])),
                  'pairs_per_evaluation': base['pairs_per_evaluation'],
                  'seconds_per_step': step_s,
                  'note': 'value = full-evaluation rate extrapolated from the '
                          'timed pairs by the marginal per-pair cost; see '
                          'measured_full_evaluations for complete, '
                          'unextrapolated evaluations of smaller particles'},
        'measured_full_evaluations': full,
        'cpu_baseline': base,
        'e2e': {'value': v, 'unit': 'evals/s', 'h2d_bytes_per_step': 0,
                'd2h_bytes_per_step': 0},
    }


def run_gcmc(torch, steps=200):
    """Grand-canonical Monte Carlo (insert / remove moves, the reference's
    rule) on a 500-atom fcc Au particle against the G(r) of a 600-atom one,
    E = 100 Rw, 1000 K, mu = 0: the O(N K) device engine against the
    reference algorithm (full energy of every trial configuration through
    Calc1D on the same GPU), same seeds, same number of steps."""
    from pyiid_gb300 import structures
    from pyiid_gb300.atoms import Atoms
    from pyiid_gb300.calc.calc_1d import Calc1D
    from pyiid_gb300.experiments.elasticscatter import ElasticScatter
    from pyiid_gb300.sim.gcmc import GrandCanonicalEnsemble
    s = ElasticScatter(exp_dict=None)
    target = s.get_pdf(Atoms(numbers=[79] * 600,
                             positions=structures.fcc_nearest(4.08, 600)))
    out = {'workload': 'GCMC, 500-atom fcc Au, Au mu = 0, 1000 K, '
                       'E = 100 Rw, insertions in a 12 A cube'}
    for name, inc in (('incremental_engine', True),
                      ('reference_algorithm', False)):
        atoms = Atoms(numbers=[79] * 500,
                      positions=structures.fcc_nearest(4.08, 500))
        atoms.set_cell(np.eye(3) * 12.0)
        atoms.set_calculator(Calc1D(target_data=target,
                                    exp_function=s.get_pdf,
                                    exp_grad_function=s.get_grad_pdf,
                                    conv=100.))
        np.random.seed(11)
        gc = GrandCanonicalEnsemble(atoms, {'Au': 0.0}, temperature=1000,
                                    seed=11, incremental=inc)
        n = steps if inc else max(steps // 10, 10)
        gc.step()
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(n):
            gc.step()
        torch.cuda.synchronize()
        dt = time.perf_counter() - t
        m = gc.metadata
        out[name] = {'moves_per_s': n / dt, 'steps_timed': n,
                     'accepted': m['accepted_additions'] + m['accepted_removals'],
                     'atoms_at_end': len(gc.traj[-1])}
    return out


def run_nuts(torch, iters=2, adapt=1):
    from pyiid_gb300 import autotune
    with autotune.variant_scope():
        return _run_nuts(torch, iters, adapt)


def _run_nuts(torch, iters, adapt):
    """NUTS on 64 chains of the 1,000-atom Au particle (300 K, E = 100 Rw,
    escape depth 6): the tree of every chain grown on the device in lock
    step, one batched exact evaluation per leapfrog step of all chains
    (pyiid_gb300.nuts.BatchedNUTS; the Debye potential is translation
    invariant, so the re-centred end point is not re-evaluated), against
    one chain of the sequential NUTSCanonicalEnsemble (the drop-in sampler
    on a Calc1D) on the same GPU."""
    from pyiid_gb300.atoms import Atoms
    from pyiid_gb300.calc.calc_1d import Calc1D
    from pyiid_gb300.experiments.elasticscatter import ElasticScatter
    from pyiid_gb300.experiments.elasticscatter.gb300_wrap import species_of
    from pyiid_gb300.nuts import BatchedNUTS
    from pyiid_gb300.sampling import PDFPotential
    from pyiid_gb300.sim.nuts_hmc import NUTSCanonicalEnsemble
    from pyiid_gb300 import structures
    s = ElasticScatter(exp_dict=None)
    ref = structures.fcc_nearest(4.08, 1000)
    target = s.get_pdf(Atoms(numbers=[79] * 1000, positions=ref))
    starts = np.stack([structures.displaced(ref, 0.05, 4 + c)
                       for c in range(64)])
    probe = Atoms(numbers=[79] * 1000, positions=starts[0])
    s._ensure(probe)
    tab = species_of(probe, 'PDF')[1]
    pot = PDFPotential([79] * 1000, target, None, conv=100., n_configs=64,
                       table=tab)
    from pyiid_gb300 import autotune
    x0 = torch.as_tensor(starts.reshape(-1, 3).astype(np.float32),
                         device='cuda')
    autotune.tune_call(lambda: pot.evaluate(x0), reps=2)
    out = {'workload': 'NUTS, 64 chains x 1000-atom fcc Au, 300 K, '
                       'E = 100 Rw, escape depth 6'}
    t = time.perf_counter()
    bn = BatchedNUTS(pot, starts, temperature=300, seeds=range(64),
                     escape_level=6, exact=False)
    bn.step(adapt)  # warm-up (graph capture, first adaptation)
    torch.cuda.synchronize()
    e = bn.engine
    step_adapted = float(e.step.median())
    lf0, ev0, acc0 = int(e.leapfrogs.sum()), e.evaluations, int(
        e.accepted.sum())
    t1 = time.perf_counter()
    ticks = bn.step(iters)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t1
    leaves = int(e.leapfrogs.sum()) - lf0
    out['batched'] = {'chain_iterations_per_s': 64 * iters / dt,
                      'leapfrog_steps_per_s': leaves / dt,
                      'accepted_samples_per_s':
                          (int(e.accepted.sum()) - acc0) / dt,
                      'timed_iterations_per_chain': iters,
                      'adaptation_iterations_before': adapt,
                      'step_size_median': {
                          'after_adaptation': step_adapted,
                          'end': float(e.step.median())},
                      'acceptance_note': (
                          'the acceptance statistic of each leaf is taken '
                          'against the previous leaf and the slice test '
                          'against the start of the iteration, as the '
                          "reference's buildtree does; dual averaging "
                          'then holds the per-step energy error near the '
                          'target while the trajectory drifts from the '
                          'start, and here no leaf passes the slice test '
                          'within the escape depth (the throughput figures '
                          'do not depend on it)'),
                      'ticks': ticks, 'ms_per_tick': 1e3 * dt / max(ticks, 1),
                      'chain_utilisation': leaves / max(64 * ticks, 1),
                      'batched_evaluations': e.evaluations - ev0,
                      'setup_s': t1 - t,
                      'tree': 'on the device (lock step, masks), '
                              'no per-leaf host exchange'}
    atoms = Atoms(numbers=[79] * 1000, positions=starts[0])
    atoms.set_calculator(Calc1D(target_data=target, exp_function=s.get_pdf,
                                exp_grad_function=s.get_grad_pdf, conv=100.))
    ens = NUTSCanonicalEnsemble(atoms, temperature=300, seed=0,
                                escape_level=6)
    t1 = time.perf_counter()
    ens.run(1)
    dt = time.perf_counter() - t1
    out['sequential_one_chain'] = {
        'chain_iterations_per_s': 1 / dt,
        'leapfrog_steps_per_s': ens.metadata['leapfrog_steps'] / dt}
    return out


WORKLOADS = {
    'fq_grad_au1000': lambda torch, **kw: run_fq_grad_au1000(torch, **kw),
    'pdf_transforms_au1000':
        lambda torch, **kw: run_pdf_transforms(torch, **kw),
    'batched_fq_256_alloys': lambda torch, **kw: run_batched(torch, **kw),
    'hmc_64_chains_au1000': lambda torch, **kw: run_hmc(torch, **kw),
    'delayed_acceptance_au1000':
        lambda torch, **kw: run_delayed_acceptance(torch, **kw),
    'delayed_acceptance_single_atom_au1000':
        lambda torch, **kw: run_delayed_acceptance_single_atom(torch, **kw),
    'exact_incremental_mh':
        lambda torch, **kw: run_incremental_mh(torch, **kw),
    'surrogate_forces_au1000x64':
        lambda torch, **kw: run_surrogate_forces(torch, **kw),
    'gcmc_au500': lambda torch, **kw: run_gcmc(torch, **kw),
    'nuts_64_chains_au1000': lambda torch, **kw: run_nuts(torch, **kw),
}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=10)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--cpu-seconds', type=float, default=15.0)
    ap.add_argument('--n-atoms', type=int, default=N_ATOMS,
                    help='particle size (default: the 20,000-atom workload; '
                         'smaller sizes are for profiling)')
    ap.add_argument('--no-cpu', action='store_true',
                    help='skip the CPU baseline sample')
    ap.add_argument('--no-workloads', action='store_true',
                    help='skip the batched and HMC secondary workloads')
    ap.add_argument('--shard-particle', action='store_true',
                    help='split the one particle across the ranks (strong '
                         'scaling) instead of running replicas')
    ap.add_argument('--no-tune', action='store_true',
                    help='use the default launch shapes (no autotuning)')
    ap.add_argument('--only-workload', default=None,
                    choices=sorted(WORKLOADS),
                    help='run one secondary workload alone and print its '
                         'result (for profiling)')
    ap.add_argument('--workload-steps', type=int, default=None,
                    help='steps of --only-workload exact_incremental_mh')
    ap.add_argument('--variant', action='append', default=[],
                    metavar='KERNEL=INDEX',
                    help='launch variant for --only-workload (e.g. mlp=1: '
                         'the tcgen05 surrogate MLP); repeatable')
    args = ap.parse_args()
    if args.only_workload:
        import torch
        from pyiid_gb300._native import context, KERNELS
        fn = WORKLOADS[args.only_workload]
        kw = {}
        if args.workload_steps and args.only_workload == 'exact_incremental_mh':
            kw['n_steps'] = args.workload_steps
        chosen = {}
        for v in args.variant:
            kern, _, idx = v.partition('=')
            if kern not in KERNELS or not idx.lstrip('-').isdigit():
                ap.error(f'--variant {v}: expected one of {sorted(KERNELS)}'
                         '=INDEX')
            context().set_variant(kern, int(idx))
            chosen[kern] = int(idx)
        out = fn(torch, **kw)
        if chosen:
            out['variants_set'] = chosen
        print(json.dumps({args.only_workload: out}))
        return
    rank, world, local = dist_env()
    if args.impl == 'reference':
        line = run_reference(args, rank, world)
    else:
        run = run_gpu_sharded if args.shard_particle else run_gpu
        line = run(args, rank, world, local)
        if line is not None and world == 1 and not args.no_cpu:
            from oracle import build_oracle
            build_oracle.build()
            line['cpu_baseline'] = cpu_sample(target_s=args.cpu_seconds,
                                              n_atoms=args.n_atoms)
    if line is not None:
        print(json.dumps(line))


if __name__ == '__main__':
    main()
