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


# ------------------------------------------------- compositions (FP64 chain)
def fq_all_bins(pos, species, ftab, qbin):
    """F(Q) [K] from Q = 0: 2 nan_to_num(S / na) with S from the C pair
    sums on every bin and na = N mean f_a f_b (flat_multi_cpu_wrap.py:44-60)."""
    from . import debye_np
    tab = np.asarray(ftab, np.float32)
    s = pair_sums(pos, species, tab, qbin, np.arange(tab.shape[1]))
    na = debye_np.normalization(tab[np.asarray(species)])
    with np.errstate(all='ignore'):
        return 2 * np.nan_to_num(s / na)


def potential_chain(pos, species, ftab, exp, qbin, gobs, kind='rw'):
    """(value, scale, gcalc, F, T) of one configuration on the PDF grid:
    F from fq_all_bins, G = F T (the FFT transform as its exact linear map,
    master_kernel.py:39-203), then get_rw / get_chi_sq
    (master_kernel.py:206-266)."""
    from . import debye_np
    f = fq_all_bins(pos, species, ftab, qbin)
    T = debye_np.tmatrix(len(f), exp['rstep'], qbin, debye_np.r_grid(exp),
                         exp['qmin'])
    gcalc = f @ T
    gobs = np.asarray(gobs, np.float64)
    fn = debye_np.get_rw if kind == 'rw' else debye_np.get_chi_sq
    val, scale = fn(gobs, gcalc)
    return val, scale, gcalc, f, T


def true_grad_rows(pos, species, ftab, exp, qbin, gobs, atoms, kind='rw',
                   with_chain=False):
    """Exact d(potential)/dx of the given atoms, [len(atoms), 3] (FP64):
    sum_k w_k dF_k/dx_a with w = T c, c the adjoint vector of the potential
    (the derivative get_grad_rw / get_grad_chi_sq contract,
    master_kernel.py:293-376) and dF = 2 dS / na from oracle_grad_rows."""
    from . import debye_np
    val, scale, gcalc, f, T = potential_chain(pos, species, ftab, exp, qbin,
                                              gobs, kind)
    c = debye_np.potential_adjoint_vector(np.asarray(gobs, np.float64),
                                          gcalc, kind)
    w = T @ c
    tab = np.asarray(ftab, np.float32)
    ds = grad_rows(pos, species, tab, qbin, atoms)
    na = debye_np.normalization(tab[np.asarray(species)])
    with np.errstate(all='ignore'):
        df = np.nan_to_num(2 * ds / na)
    if with_chain:
        return df @ w, (val, scale, gcalc, f, T)
    return df @ w


def moved_atom_sums(pos, species, ftab, qbin, atom, new_xyz):
    """S(x') - S(x) in FP64 when ``atom`` moves to ``new_xyz`` (float64,
    not rounded to float32): the atom's N - 1 pair terms before and after."""
    x = np.asarray(pos, np.float32).astype(np.float64)
    tab = np.asarray(ftab, np.float64)
    sp = np.asarray(species)
    k = tab.shape[1]
    q = np.arange(k) * float(qbin)
    others = np.arange(len(x)) != atom
    fb = tab[sp[others]] * tab[sp[atom]][None]

    def terms(xa):
        r = np.linalg.norm(x[others] - xa[None], axis=1)
        return (fb * np.sin(np.outer(r, q)) / r[:, None]).sum(0)
    return terms(np.asarray(new_xyz, np.float64)) - terms(x[atom])
