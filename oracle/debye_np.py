"""FP64 NumPy restatement of pyIID's elastic-scattering path (test oracle).

TEST INFRASTRUCTURE ONLY.  This module is the parity checker for the GB300
kernels: only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of ``bench.py`` may import it.  The product (``pyiid_gb300``) never calls it.

Every function restates the reference algorithm in float64 arithmetic on the
float32 positions the reference itself uses (``astype(np.float32)``,
cpu_wrappers/flat_multi_cpu_wrap.py:22-29), so it is the exact value the
reference's float32 code approximates.  Citations are paths inside the
pyIID source tree (``pyiid/...``).

Pinning: ``tests/test_oracle_golden.py`` checks this module against vectors
produced by running the reference's own Python code (numba JIT disabled, as
its CI's NUMBA_DISABLE_JIT leg does; see ``tests/golden/make_golden.py``) and
against the reference's known-answer tests
(pyiid/tests/test_master/test_master_kernel.py:19-48).
"""
import math

import numpy as np

__all__ = [
    'DEFAULT_EXP', 'update_experiment', 'pdf_qbin', 'scatter_vector', 'r_grid',
    'wrap_atoms_tables', 'pair_sums', 'normalization', 'fq', 'grad_fq',
    'pdf_fft', 'pdf_tmatrix', 'tmatrix', 'grad_pdf', 'get_rw', 'get_chi_sq',
    'get_scale', 'get_grad_rw', 'get_grad_chi_sq', 'potential_adjoint_vector',
    'true_grad_potential', 'sq', 'iq',
]

# pyiid/experiments/elasticscatter/__init__.py:86-89
DEFAULT_EXP = {'qmin': 0.0, 'qmax': 25, 'qbin': .1, 'rmin': 0.0,
               'rmax': 40.0, 'rstep': .01, 'sampling': 'full'}


def update_experiment(exp_dict=None):
    """Defaults, Nyquist sampling and PDF grid step.

    pyiid/experiments/elasticscatter/__init__.py:180-204.
    """
    exp = dict(exp_dict or {})
    for k, v in DEFAULT_EXP.items():
        exp.setdefault(k, v)
    if exp['sampling'] == 'ns':
        exp['rstep'] = np.pi / exp['qmax']
    return exp


def pdf_qbin(exp):
    """pyiid/experiments/elasticscatter/__init__.py:203-204."""
    return np.pi / (exp['rmax'] + 6 * 2 * np.pi / exp['qmax'])


def scatter_vector(exp, pdf=False):
    """pyiid/experiments/elasticscatter/__init__.py:526-547."""
    if pdf:
        q = pdf_qbin(exp)
        return np.arange(0., math.floor(exp['qmax'] / q) * q, q)
    return np.arange(exp['qmin'],
                     math.floor(exp['qmax'] / exp['qbin']) * exp['qbin'],
                     exp['qbin'])


def r_grid(exp):
    """pyiid/experiments/elasticscatter/__init__.py:549-558."""
    return np.arange(exp['rmin'], exp['rmax'], exp['rstep'])


def wrap_atoms_tables(numbers, exp, form_factor):
    """Per-atom scatter arrays exactly as ``_wrap_atoms`` builds them.

    pyiid/experiments/elasticscatter/__init__.py:110-151 with
    kernels/master_kernel.py:14-36.  Reproduces two reference behaviours:
    both grids are evaluated at ``k * exp['qbin']`` (line 137), and row i of
    the element table is evaluated for ``numbers[i]`` (the i-th atom) but
    assigned to element ``list(set(numbers))[i]`` (lines 123-143).
    ``form_factor(Z, s)`` stands for xraylib.FF_Rayl with s = Q / (4 pi).
    Returns (fq_table [N, K], pdf_table [N, K']) as float32.
    """
    numbers = np.asarray(numbers)
    n = len(numbers)
    e_list = list(set(numbers.tolist()))
    out = []
    for qbin in (exp['qbin'], pdf_qbin(exp)):
        qmax_bin = int(math.floor(exp['qmax'] / qbin))
        set_arr = np.zeros((len(e_list), qmax_bin), dtype=np.float32)
        for kq in range(qmax_bin):
            for tx in range(len(e_list)):
                set_arr[tx, kq] = form_factor(int(numbers[tx]),
                                              kq * exp['qbin'] / 4 / np.pi)
        arr = np.zeros((n, qmax_bin), dtype=np.float32)
        for i in range(len(e_list)):
            arr[np.where(numbers == e_list[i])[0], :] = set_arr[i, :]
        out.append(arr)
    return out[0], out[1]


def _pairs(n):
    i, j = np.tril_indices(n, -1)  # i > j, ordered like k_to_ij
    return i, j


def _pos64(pos, cast32):
    """Positions as FP64; rounded through float32 first (as the reference
    casts them) unless cast32 is False (finite-difference checks)."""
    if cast32:
        return np.asarray(pos, dtype=np.float32).astype(np.float64)
    return np.asarray(pos, dtype=np.float64)


def pair_sums(pos, scatter, qbin, chunk=20000, cast32=True):
    """S_k = sum_{i>j} f_i f_j sin(Q_k r_ij) / r_ij in FP64.

    kernels/cpu_flat.py:16-114 (d, r, norm, omega, fq) summed over pairs as
    cpu_wrappers/flat_serial_cpu_wrap.py:61.  Q_k = k * qbin.
    """
    q = _pos64(pos, cast32)
    f = np.asarray(scatter, dtype=np.float64)
    n, kmax = f.shape
    Q = np.arange(kmax) * float(qbin)
    i, j = _pairs(n)
    out = np.zeros(kmax)
    with np.errstate(all='ignore'):
        for s in range(0, len(i), chunk):
            ii, jj = i[s:s + chunk], j[s:s + chunk]
            r = np.sqrt(((q[ii] - q[jj]) ** 2).sum(1))
            out += (f[ii] * f[jj] * np.sin(Q[None] * r[:, None])
                    / r[:, None]).sum(0)
    return out


def normalization(scatter):
    """na_k = N * mean_{i>j} f_i f_j (flat_multi_cpu_wrap.py:52-54), FP64."""
    f = np.asarray(scatter, dtype=np.float64)
    n = f.shape[0]
    if n < 2:
        return np.full(f.shape[1], np.nan)
    tot = f.sum(0)
    sq = (f * f).sum(0)
    pairsum = (tot * tot - sq) / 2
    return n * pairsum / (n * (n - 1) / 2)


def fq(pos, scatter, qbin, cast32=True):
    """F(Q) from Q = 0 (the plug-in's return value before slicing).

    2 * nan_to_num(S / na): cpu_wrappers/flat_multi_cpu_wrap.py:44-60.
    """
    s = pair_sums(pos, scatter, qbin, cast32=cast32)
    with np.errstate(all='ignore'):
        return 2 * np.nan_to_num(s / normalization(scatter))


def grad_fq(pos, scatter, qbin, convention='reference', chunk=20000,
            cast32=True):
    """Gradient of F(Q), [N, 3, K].

    'reference': -(1/na) dS/dx (= -1/2 dF/dx), the value of wrap_fq_grad
    (kernels/cpu_flat.py:122-194, kernels/cpu_experimental.py:8-15,
    cpu_wrappers/flat_serial_cpu_wrap.py:124-133).  'true': dF/dx.
    """
    q = _pos64(pos, cast32)
    f = np.asarray(scatter, dtype=np.float64)
    n, kmax = f.shape
    Q = np.arange(kmax) * float(qbin)
    out = np.zeros((n, 3, kmax))
    i, j = _pairs(n)
    with np.errstate(all='ignore'):
        for s in range(0, len(i), chunk):
            ii, jj = i[s:s + chunk], j[s:s + chunk]
            d = q[ii] - q[jj]
            r = np.sqrt((d ** 2).sum(1))[:, None]
            qr = Q[None] * r
            a = (Q[None] * np.cos(qr) - np.sin(qr) / r) / r ** 2
            g = (f[ii] * f[jj] * a)[:, None, :] * d[:, :, None]
            np.add.at(out, ii, -g)
            np.add.at(out, jj, g)
        out = np.nan_to_num(out / normalization(scatter))
    if convention == 'true':
        out = -2 * out
    return out


def sq(fq_sliced, exp):
    """pyiid/experiments/elasticscatter/__init__.py:393-420."""
    with np.errstate(all='ignore'):
        s = fq_sliced / scatter_vector(exp) + 1.0
    s[np.isinf(s)] = 0.
    return s


def iq(sq_v, fq_table, exp):
    """pyiid/experiments/elasticscatter/__init__.py:422-446."""
    f2 = np.average(fq_table, axis=0) ** 2
    return sq_v * f2[int(np.floor(exp['qmin'] / exp['qbin'])):]


# ----------------------------------------------------------------- G(r)
def _fft_gr_to_fq(g, rstep, rmin):
    """kernels/master_kernel.py:131-203."""
    padrmin = int(round(rmin / rstep))
    npad1 = padrmin + len(g)
    npad2 = (1 << int(math.ceil(math.log(npad1, 2)))) * 2
    npad4 = 4 * npad2
    gpadc = np.zeros(npad4)
    gpadc[:2 * len(g):2] = g[:]
    gpadc[-2:-2 * len(g) + 1:-2] = -1 * g[1:]
    gpadcfft = np.fft.ifft(gpadc)
    f = np.zeros(npad2, dtype=complex)
    f[:] = gpadcfft[:npad2 * 2:2] * npad2 * rstep
    return f.imag


def pdf_fft(fpad, rstep, qstep, rgrid, qmin):
    """get_pdf_at_qmin, kernels/master_kernel.py:39-128 (FFT form)."""
    fpad = np.array(fpad, dtype=np.float64)
    fpad[:int(math.ceil(qmin / qstep))] = 0.0
    nfromdr = int(math.ceil(math.pi / rstep / qstep))
    if nfromdr > int(len(fpad)):
        fpad2 = np.zeros(nfromdr)
        fpad2[:len(fpad)] = fpad
        fpad = fpad2
    gpad = _fft_gr_to_fq(fpad, qstep, qmin) * 2.0 / math.pi
    drpad = math.pi / (len(gpad) * qstep)
    axdrp = rgrid / drpad / 2
    aiplo = axdrp.astype(int)
    aiphi = aiplo + 1
    awphi = axdrp - aiplo
    awplo = 1.0 - awphi
    return (awplo * gpad[aiplo] + awphi * gpad[aiphi]) * 2


def tmatrix(n_bins, rstep, qstep, rgrid, qmin):
    """The FFT form of get_pdf_at_qmin written as G = F @ T, T [K, R].

    With npad2 as in fft_gr_to_fq the odd-extended inverse FFT equals
    gpad[i] = (qstep/pi) sum_m F_m sin(2 pi m i / npad2); linear
    interpolation then gives
    T[m, i] = (2 qstep/pi)((1-w) sin(2 pi m lo/npad2) + w sin(2 pi m (lo+1)/npad2)).
    """
    kz = int(math.ceil(qmin / qstep))
    nfromdr = int(math.ceil(math.pi / rstep / qstep))
    length = max(n_bins, nfromdr)
    padrmin = int(round(qmin / qstep))
    npad2 = (1 << int(math.ceil(math.log(padrmin + length, 2)))) * 2
    drpad = math.pi / (npad2 * qstep)
    x = np.asarray(rgrid) / drpad / 2
    lo = x.astype(np.int64)
    w = x - lo
    m = np.arange(n_bins, dtype=np.int64)[:, None]
    sa = np.sin(2 * np.pi * ((m * lo[None]) % npad2) / npad2)
    sb = np.sin(2 * np.pi * ((m * (lo[None] + 1)) % npad2) / npad2)
    T = 2 * qstep / np.pi * ((1 - w)[None] * sa + w[None] * sb)
    T[:max(kz, 0)] = 0.0
    return T


def pdf_tmatrix(fq_full, rstep, qstep, rgrid, qmin):
    return np.asarray(fq_full, dtype=np.float64) @ tmatrix(
        len(fq_full), rstep, qstep, rgrid, qmin)


def grad_pdf(grad_fq_ref, rstep, qstep, rgrid, qmin):
    """kernels/master_kernel.py:276-290: the transform of every [a, c] row."""
    g = np.asarray(grad_fq_ref, dtype=np.float64)
    T = tmatrix(g.shape[-1], rstep, qstep, rgrid, qmin)
    return g @ T


# ------------------------------------------------------------ potentials
def get_scale(target, calculated):
    """kernels/master_kernel.py:388-389."""
    return np.dot(calculated.T, target) / np.dot(calculated.T, calculated)


def get_rw(gobs, gcalc, weight=None):
    """kernels/master_kernel.py:206-236."""
    if weight is None:
        weight = np.ones(gcalc.shape)
    with np.errstate(all='ignore'):
        scale = get_scale(gobs, gcalc)
    if scale <= 0:
        return 1, 1
    top = np.sum(weight * (gobs - scale * gcalc) ** 2)
    bottom = np.sum(weight * gobs ** 2)
    return np.sqrt(top / bottom).real, scale


def get_chi_sq(gobs, gcalc):
    """kernels/master_kernel.py:239-266."""
    with np.errstate(all='ignore'):
        scale = get_scale(gobs, gcalc)
    if scale <= 0:
        scale = 1
    return np.sum((gobs - scale * gcalc) ** 2), scale


def _grad_scale(gobs, gcalc, gpdf):
    """kernels/master_kernel.py:392-396, vectorised over the [N, 3] rows."""
    a = get_scale(gobs, gcalc)
    return ((-2 * a * (gpdf @ gcalc) + gpdf @ gobs)
            / np.dot(gcalc, gcalc))


def get_grad_rw(gpdf, gcalc, gobs, rw, scale):
    """kernels/master_kernel.py:293-347 (returns the [N, 3] array)."""
    gpdf = np.asarray(gpdf, dtype=np.float64)
    if scale <= 0:
        grad_a = 0
        scale = 1
    else:
        grad_a = _grad_scale(gobs, gcalc, gpdf)
    e = gobs - scale * gcalc
    return (-1 * rw / np.dot(e, e)
            * ((scale * gpdf) @ e + grad_a * np.dot(gcalc, e)))


def get_grad_chi_sq(gpdf, gcalc, gobs, scale):
    """kernels/master_kernel.py:350-376."""
    gpdf = np.asarray(gpdf, dtype=np.float64)
    grad_a = _grad_scale(gobs, gcalc, gpdf)
    if scale <= 0:
        grad_a = 0
    e = gobs - scale * gcalc
    return -2 * ((scale * gpdf) @ e + grad_a * np.dot(gcalc, e))


def potential_adjoint_vector(gobs, gcalc, potential='rw'):
    """c with d(potential) = sum_r c_r dG_r, as the two functions above
    contract it (linear in dG)."""
    a = get_scale(gobs, gcalc)
    if potential == 'rw':
        val, s = get_rw(gobs, gcalc)
        if s <= 0:
            s, ga_on = 1, 0.0
        else:
            ga_on = 1.0
        e = gobs - s * gcalc
        pre = -val / np.dot(e, e)
    else:
        val, s = get_chi_sq(gobs, gcalc)
        ga_on = 0.0 if s <= 0 else 1.0
        e = gobs - s * gcalc
        pre = -2.0
    dscale = (gobs - 2 * a * gcalc) / np.dot(gcalc, gcalc)
    return pre * (s * e + ga_on * np.dot(gcalc, e) * dscale)


def potential_value(pos, pdf_table, exp, gobs, potential='rw', cast32=True):
    """Rw or chi^2 of one configuration on the PDF grid (FP64)."""
    qb = pdf_qbin(exp)
    gcalc = pdf_tmatrix(fq(pos, pdf_table, qb, cast32=cast32), exp['rstep'],
                        qb, r_grid(exp), exp['qmin'])
    if potential == 'rw':
        return get_rw(gobs, gcalc)[0]
    return get_chi_sq(gobs, gcalc)[0]


def true_grad_potential(pos, pdf_table, exp, gobs, potential='rw'):
    """Exact d(potential)/d(positions) through F -> G -> potential (FP64).

    Equals -2 x the reference's wrap_grad_rw(get_grad_pdf(atoms), ...)
    (calc/__init__.py:56-105), i.e. the gradient without the reference's
    factor 1/2.
    """
    qb = pdf_qbin(exp)
    rg = r_grid(exp)
    fqv = fq(pos, pdf_table, qb)
    gcalc = pdf_tmatrix(fqv, exp['rstep'], qb, rg, exp['qmin'])
    c = potential_adjoint_vector(gobs, gcalc, potential)
    gq = grad_fq(pos, pdf_table, qb, convention='true')
    T = tmatrix(gq.shape[-1], exp['rstep'], qb, rg, exp['qmin'])
    w = T @ c
    if potential == 'rw':
        val = get_rw(gobs, gcalc)[0]
    else:
        val = get_chi_sq(gobs, gcalc)[0]
    return val, gq @ w
