"""ctypes wrapper of oracle/debye_ref.c (test infrastructure only)."""
import ctypes

import numpy as np

from . import build_oracle

_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build_oracle.build())
        _lib.port_fq_grad_tasks.restype = ctypes.c_int
        _lib.port_fq_grad_tasks.argtypes = [
            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
            ctypes.c_double, ctypes.c_long, ctypes.c_long, ctypes.c_void_p,
            ctypes.c_void_p, ctypes.c_int]
        for name in ('oracle_pair_sums', 'oracle_grad_rows'):
            fn = getattr(_lib, name)
            fn.restype = None
            fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                           ctypes.c_void_p, ctypes.c_int, ctypes.c_double,
                           ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        _lib.port_fq_allocation.restype = ctypes.c_long
        _lib.port_fq_allocation.argtypes = [ctypes.c_long, ctypes.c_long,
                                            ctypes.c_double]
        _lib.port_grad_allocation.restype = ctypes.c_long
        _lib.port_grad_allocation.argtypes = [ctypes.c_long, ctypes.c_long,
                                              ctypes.c_double]
    return _lib


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def pair_sums(pos, species, ftab, qbin, bins):
    """FP64 S_k on the requested bins (see oracle_pair_sums)."""
    pos, sp, tab = _c(pos, np.float32), _c(species, np.int32), _c(ftab, np.float32)
    bins = _c(bins, np.int32)
    out = np.zeros(len(bins))
    lib().oracle_pair_sums(pos.ctypes.data, sp.ctypes.data, len(pos),
                           tab.ctypes.data, tab.shape[1], float(qbin),
                           bins.ctypes.data, len(bins), out.ctypes.data)
    return out


def grad_rows(pos, species, ftab, qbin, atoms):
    """FP64 dS/dx rows [len(atoms), 3, K] (no normalisation)."""
    pos, sp, tab = _c(pos, np.float32), _c(species, np.int32), _c(ftab, np.float32)
    atoms = _c(atoms, np.int32)
    out = np.zeros((len(atoms), 3, tab.shape[1]))
    lib().oracle_grad_rows(pos.ctypes.data, sp.ctypes.data, len(pos),
                           tab.ctypes.data, tab.shape[1], float(qbin),
                           atoms.ctypes.data, len(atoms), out.ctypes.data)
    return out


def port_tasks(pos, per_atom_scatter, qbin, chunk, n_pairs, want_fq=True,
               want_grad=True, n_threads=0):
    """FP32 port of the reference CPU path over pairs [0, n_pairs).

    Returns (task sums [K] FP64 or None, summed task gradients [n,3,K] f32 or
    None, threads used).
    """
    q = _c(pos, np.float32)
    scat = _c(per_atom_scatter, np.float32)
    n, k = scat.shape
    sums = np.zeros(k) if want_fq else None
    grad = np.zeros((n, 3, k), np.float32) if want_grad else None
    used = lib().port_fq_grad_tasks(
        q.ctypes.data, scat.ctypes.data, n, k, float(qbin), int(chunk),
        int(n_pairs), sums.ctypes.data if want_fq else None,
        grad.ctypes.data if want_grad else None, int(n_threads))
    return sums, grad, used


def port_fq(pos, per_atom_scatter, qbin, chunk=4096, n_threads=0):
    """Full reference-path F(Q) via the port (flat_multi_cpu_wrap.wrap_fq)."""
    n = len(pos)
    sums, _, _ = port_tasks(pos, per_atom_scatter, qbin, chunk,
                            n * (n - 1) // 2, True, False, n_threads)
    final = sums.astype(np.float32)
    scat = np.asarray(per_atom_scatter, np.float32)
    i, j = np.tril_indices(n, -1)
    na = np.mean(scat[i] * scat[j], axis=0, dtype=np.float32) * np.float32(n)
    with np.errstate(all='ignore'):
        return 2 * np.nan_to_num(final / na)
