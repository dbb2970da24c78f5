"""GPU-backed versions of the reference's master_kernel functions.

Same names, arguments and return conventions as
pyiid/experiments/elasticscatter/kernels/master_kernel.py; arithmetic runs in
the sm_103a library (pyiid_pdf / pyiid_potential / pyiid_potential_grad).
"""
import numpy as np
import torch

from .... import debye
from ....scatter_factors import form_factor

__all__ = ['get_scatter_array', 'get_pdf_at_qmin', 'get_rw', 'get_chi_sq',
           'get_grad_rw', 'get_grad_chi_sq', 'get_scale', 'get_grad_scale',
           'grad_pdf']


def get_scatter_array(scatter_array, numbers, qbin):
    """Fill [n, K] with f(numbers[tx], kq*qbin/4pi) (master_kernel.py:14-36),
    using the stand-in form factor of pyiid_gb300.scatter_factors."""
    n, qmax_bin = scatter_array.shape
    for kq in range(qmax_bin):
        for tx in range(n):
            scatter_array[tx, kq] = form_factor(int(numbers[tx]),
                                                kq * qbin / 4 / np.pi)


def _dev(a, dtype):
    return torch.as_tensor(np.ascontiguousarray(a, dtype=dtype), device='cuda')


def get_pdf_at_qmin(fpad, rstep, qstep, rgrid, qmin):
    """G(r) from F(Q) (master_kernel.py:39-105); float64 [len(rgrid)].

    Like the reference, bins below ceil(qmin/qstep) of ``fpad`` are zeroed
    in place."""
    import math
    fpad[:int(math.ceil(qmin / qstep))] = 0.0
    g = debye.pdf(_dev(fpad, np.float32), qstep, rstep, rgrid, qmin)
    return g.cpu().numpy()


def grad_pdf(grad_fq, rstep, qstep, rgrid, qmin):
    """master_kernel.py:276-290 on the GPU."""
    g = _dev(grad_fq, np.float32)
    return debye.grad_pdf(g, qstep, rstep, rgrid, qmin).cpu().numpy()


def _pot(gobs, gcalc, kind, weight=None):
    w = None if weight is None else _dev(weight, np.float64)
    out = debye.potential(_dev(gobs, np.float64), _dev(gcalc, np.float64),
                          kind, weight=w).cpu().numpy()
    return out


def get_rw(gobs, gcalc, weight=None):
    """(Rw, scale); (1, 1) for a non-positive scale (master_kernel.py:206-236).
    ``weight`` weighs the residual and the normalisation point by point; the
    scale is the unweighted one, as in the reference."""
    if weight is not None:
        weight = np.array(np.broadcast_to(np.asarray(weight, np.float64),
                                          np.shape(gcalc)))
    v, s = _pot(gobs, gcalc, 'rw', weight)
    if s == 1.0 and v == 1.0:
        return 1, 1
    return v, s


def get_chi_sq(gobs, gcalc):
    """(chi^2, scale) (master_kernel.py:239-266)."""
    v, s = _pot(gobs, gcalc, 'chi_sq')
    return v, s


def get_scale(target, calculated):
    """master_kernel.py:388-389 (host dot products of two [R] vectors)."""
    return np.dot(calculated.T, target) / np.dot(calculated.T, calculated)


def get_grad_scale(target, calculated, grad_calculated, tx, tz):
    """master_kernel.py:392-396."""
    a = get_scale(target, calculated)
    g = grad_calculated[tx, tz, :]
    return (-2 * a * np.dot(calculated, g) + np.dot(target, g)) / np.dot(
        calculated, calculated)


def _grad(grad_out, grad_pdf_arr, gcalc, gobs, kind):
    g = debye.potential_grad(_dev(grad_pdf_arr, np.float64),
                             _dev(gcalc, np.float64), _dev(gobs, np.float64),
                             kind).cpu().numpy()
    grad_out[...] = g
    return grad_out


def get_grad_rw(grad_rw, grad_pdf, gcalc, gobs, rw, scale):
    """Fill grad_rw [N, 3] (master_kernel.py:293-347).  rw and scale are
    recomputed on the device from (gcalc, gobs), which is what every
    reference caller passes (calc/__init__.py:76-78)."""
    return _grad(grad_rw, grad_pdf, gcalc, gobs, 'rw')


def get_grad_chi_sq(grad_rw, grad_pdf, gcalc, gobs, scale):
    """Fill grad_rw [N, 3] (master_kernel.py:350-376)."""
    return _grad(grad_rw, grad_pdf, gcalc, gobs, 'chi_sq')
