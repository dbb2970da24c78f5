"""``FQCalc(obs_data, scatter, conv, potential)``: the F(Q)-space counterpart
of PDFCalc; a Calc1D on get_fq/get_grad_fq."""
from .calc_1d import Calc1D

__all__ = ['FQCalc']


class FQCalc(Calc1D):
    def __init__(self, obs_data=None, scatter=None, conv=1., potential='rw',
                 **kwargs):
        Calc1D.__init__(self, target_data=obs_data,
                        exp_function=scatter.get_fq,
                        exp_grad_function=scatter.get_grad_fq, conv=conv,
                        potential=potential, **kwargs)
