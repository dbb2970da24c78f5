"""``PDFCalc(obs_data, scatter, conv, potential)``: the pre-Calc1D name used by
pyiid's benchmarks/time_comparison.py:6,45; a Calc1D on get_pdf/get_grad_pdf."""
from .calc_1d import Calc1D

__all__ = ['PDFCalc']


class PDFCalc(Calc1D):
    def __init__(self, obs_data=None, scatter=None, conv=1., potential='rw',
                 **kwargs):
        Calc1D.__init__(self, target_data=obs_data,
                        exp_function=scatter.get_pdf,
                        exp_grad_function=scatter.get_grad_pdf, conv=conv,
                        potential=potential, **kwargs)
