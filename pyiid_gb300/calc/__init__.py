"""Rw / chi^2 potentials and their gradients (pyiid/calc/__init__.py:10-105).

Same names and signatures; the arithmetic runs in the sm_103a library.
"""
import numpy as np

from ..experiments.elasticscatter.kernels.master_kernel import (
    get_rw, get_chi_sq, get_grad_rw, get_grad_chi_sq)

__all__ = ['wrap_rw', 'wrap_chi_sq', 'wrap_grad_rw', 'wrap_grad_chi_sq']


def wrap_rw(gcalc, gobs):
    """(Rw, scale) of calculated vs observed 1D data."""
    rw, scale = get_rw(gobs, gcalc, weight=None)
    return rw, scale


def wrap_chi_sq(gcalc, gobs):
    """(chi^2, scale) of calculated vs observed 1D data."""
    rw, scale = get_chi_sq(gobs, gcalc)
    return rw, scale


def wrap_grad_rw(grad_gcalc, gcalc, gobs):
    """Gradient of Rw w.r.t. positions from the gradient of the 1D data."""
    rw, scale = wrap_rw(gcalc, gobs)
    grad_rw = np.zeros((len(grad_gcalc), 3))
    get_grad_rw(grad_rw, grad_gcalc, gcalc, gobs, rw, scale)
    return grad_rw


def wrap_grad_chi_sq(grad_gcalc, gcalc, gobs):
    """Gradient of chi^2 w.r.t. positions from the gradient of the 1D data."""
    chi_sq, scale = wrap_chi_sq(gcalc, gobs)
    grad_chi_sq = np.zeros((len(grad_gcalc), 3))
    get_grad_chi_sq(grad_chi_sq, grad_gcalc, gcalc, gobs, scale)
    return grad_chi_sq
