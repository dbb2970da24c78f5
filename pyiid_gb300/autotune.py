"""Autotuner for the pair-kernel launch shapes.

The F(Q) and dF/dx kernels exist in several launch shapes (bins per thread,
pairs interleaved per thread, threads per CTA; see ``pyiid_variant_info``).
:func:`tune` times every variant on the caller's own problem with CUDA
events, selects the fastest on the device context, and remembers the choice
in a JSON cache keyed by (device, kernel, atom-count bucket, bins, species),
so :func:`apply_cached` can restore it without timing.

The cache lives at ``$PYIID_GB300_TUNE_CACHE`` or
``~/.cache/pyiid_gb300/tuning.json``.
"""
import ctypes
import json
import os

import numpy as np
import torch

from . import debye
from ._native import context, load, KERNELS

__all__ = ['variants', 'tune', 'tune_call', 'variant_scope', 'apply_cached',
           'cache_path']


def cache_path():
    return os.environ.get('PYIID_GB300_TUNE_CACHE') or os.path.join(
        os.path.expanduser('~'), '.cache', 'pyiid_gb300', 'tuning.json')


def variants(kernel):
    """[(index, {'bins_per_thread', 'pairs_per_thread', 'threads'})]"""
    lib = load()
    out = []
    for i in range(lib.pyiid_variant_count(KERNELS[kernel])):
        p = (ctypes.c_int32 * 3)()
        lib.pyiid_variant_info(KERNELS[kernel], i, p, 3)
        out.append((i, {'bins_per_thread': p[0], 'pairs_per_thread': p[1],
                        'threads': p[2]}))
    return out


def _key(kernel, n_atoms, n_bins, n_species):
    dev = torch.cuda.get_device_name()
    bucket = 1 << max(0, int(np.ceil(np.log2(max(n_atoms, 1)))))
    return f'{dev}|{kernel}|N<={bucket}|K{n_bins}|S{n_species}'


def _load_cache():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save_cache(c):
    p = cache_path()
    try:
        os.makedirs(os.path.dirname(p), exist_ok=True)
        tmp = p + f'.{os.getpid()}'
        with open(tmp, 'w') as f:
            json.dump(c, f, indent=1, sort_keys=True)
        os.replace(tmp, p)
    except OSError:
        pass


def _time(fn, reps):
    fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        s.record()
        fn()
        e.record()
        e.synchronize()
        ts.append(s.elapsed_time(e))
    return float(np.median(ts))


def tune(positions, species, scatter, qbin, k_begin=0,
         kernels=('fq', 'grad_fq'), reps=3, save=True):
    """Time all variants of ``kernels`` on this problem, select the fastest.

    Returns {kernel: {'best': index, 'ms': {index: median ms}}}.
    """
    pos = debye.as_positions(positions)
    tab = np.asarray(scatter, np.float32)
    n, k = pos.shape[0], tab.shape[1]
    ctx = context(pos.device.index)
    out = torch.empty(k, dtype=torch.float32, device=pos.device)
    gout = (torch.empty((n, 3, k), dtype=torch.float32, device=pos.device)
            if 'grad_fq' in kernels else None)
    cache = _load_cache()
    result = {}
    for kern in kernels:
        if kern == 'fq':
            fn = lambda: debye.fq(pos, species, tab, qbin, k_begin, out=out)  # noqa: E731
        else:
            fn = lambda: debye.grad_fq(pos, species, tab, qbin, k_begin,  # noqa: E731
                                       out=gout)
        ms = {}
        for idx, _ in variants(kern):
            ctx.set_variant(kern, idx)
            ms[idx] = _time(fn, reps)
        best = min(ms, key=ms.get)
        ctx.set_variant(kern, best)
        result[kern] = {'best': best, 'ms': ms}
        cache[_key(kern, n, k - k_begin, tab.shape[0])] = best
    if save:
        _save_cache(cache)
    return result


def tune_call(fn, kernels=('fq', 'adjoint'), reps=3, device=None):
    """Time ``fn()`` (any workload built on the pair kernels, e.g. a batched
    PDFPotential.evaluate or batch_fq call) under every variant of
    ``kernels`` in turn, keeping the fastest of each (the kernels are tuned
    one after the other, the others at their current variant).

    Returns {kernel: {'best': index, 'ms': {index: median ms}}}."""
    ctx = context(device)
    result = {}
    for kern in kernels:
        ms = {}
        for idx, _ in variants(kern):
            ctx.set_variant(kern, idx)
            ms[idx] = _time(fn, reps)
        best = min(ms, key=ms.get)
        ctx.set_variant(kern, best)
        result[kern] = {'best': best, 'ms': ms}
    return result


class variant_scope:
    """Context manager restoring the device context's variants on exit
    (variants are per context, so tuning one workload would otherwise
    change the launch shapes of every later call)."""

    def __init__(self, device=None):
        self.ctx = context(device)

    def __enter__(self):
        self.saved = {k: self.ctx.get_variant(k) for k in KERNELS}
        return self.ctx

    def __exit__(self, *exc):
        for k, v in self.saved.items():
            self.ctx.set_variant(k, v)
        return False


def apply_cached(n_atoms, n_bins_computed, n_species, device=None):
    """Select cached variants for this problem class; returns what was set."""
    cache = _load_cache()
    ctx = context(device)
    done = {}
    for kern in ('fq', 'grad_fq'):
        v = cache.get(_key(kern, n_atoms, n_bins_computed, n_species))
        if v is not None:
            ctx.set_variant(kern, int(v))
            done[kern] = int(v)
    return done
