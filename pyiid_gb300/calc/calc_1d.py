"""ASE-style calculator for a 1D experiment (pyiid/calc/calc_1d.py:9-101).

``Calc1D(target_data, exp_function, exp_grad_function, conv, potential)``
with the reference's semantics:
  energy = conv * potential(exp_function(atoms), target)
  forces = conv * grad_potential(exp_grad_function(atoms), exp_function(atoms),
                                 target)
Because the reference's exp_grad_function returns -1/2 of the true gradient
(see ElasticScatter.get_grad_fq), these forces are -1/2 * conv * grad(E/conv);
``true_forces=True`` returns the physical -dE/dx instead.

When the two functions are ``get_pdf`` / ``get_grad_pdf`` of a GB300
ElasticScatter, energy and forces come from one fused device call
(F -> G -> potential -> adjoint gradient, no [N,3,K] or [N,3,R] arrays);
otherwise the functions are called exactly as the reference does.
"""
import numpy as np

from ..atoms import Calculator
from . import wrap_rw, wrap_chi_sq, wrap_grad_rw, wrap_grad_chi_sq

__all__ = ['Calc1D']


class Calc1D(Calculator):
    """Class for doing PDF based Rw / chi**2 calculations."""
    implemented_properties = ['energy', 'forces']

    def __init__(self, restart=None, ignore_bad_restart_file=False, label=None,
                 atoms=None, target_data=None, exp_function=None,
                 exp_grad_function=None, conv=1., potential='rw',
                 true_forces=False, **kwargs):
        Calculator.__init__(self, restart, ignore_bad_restart_file, label,
                            atoms, **kwargs)
        if target_data is None or len(target_data.shape) != 1:
            raise NotImplementedError('Need a 1d array target data set')
        if exp_function is None or exp_grad_function is None:
            raise NotImplementedError('Need functions which return the '
                                      'simulated data associated with the '
                                      'experiment and its gradient')
        self.target_data = target_data
        self.exp_function = exp_function
        self.exp_grad_function = exp_grad_function
        self.scale = 1
        self.rw_to_eV = conv
        self.true_forces = bool(true_forces)
        if potential == 'chi_sq':
            self.potential = wrap_chi_sq
            self.grad = wrap_grad_chi_sq
        elif potential == 'rw':
            self.potential = wrap_rw
            self.grad = wrap_grad_rw
        else:
            raise NotImplementedError('Potential not implemented')
        self.potential_name = potential
        self._fused = self._fused_scatter()

    def _fused_scatter(self):
        from ..experiments.elasticscatter import ElasticScatter
        f, g = self.exp_function, self.exp_grad_function
        s = getattr(f, '__self__', None)
        if (isinstance(s, ElasticScatter) and getattr(g, '__self__', None) is s
                and getattr(f, '__func__', None) is ElasticScatter.get_pdf
                and getattr(g, '__func__', None) is
                ElasticScatter.get_grad_pdf):
            return s
        return None

    def calculate(self, atoms=None, properties=['energy'],
                  system_changes=['positions', 'numbers', 'cell', 'pbc',
                                  'charges', 'magmoms']):
        Calculator.calculate(self, atoms, properties, system_changes)
        if self._fused is not None:
            self._calculate_fused(self.atoms, 'forces' in properties)
            return
        if len(system_changes) > 0:
            if 'energy' in properties:
                self.calculate_energy(self.atoms)
            if 'forces' in properties:
                self.calculate_forces(self.atoms)
        for prop in properties:
            if prop not in self.results:
                if prop == 'energy':
                    self.calculate_energy(self.atoms)
                if prop == 'forces':
                    self.calculate_forces(self.atoms)

    def _calculate_fused(self, atoms, want_forces):
        import torch
        from .. import debye
        from ..experiments.elasticscatter.gb300_wrap import species_of
        scat = self._fused
        scat._ensure(atoms)
        sp, tab = species_of(atoms, 'PDF')
        out = debye.batch_potential_grad(
            atoms.get_positions(), sp, np.array([0, len(atoms)]), tab,
            scat.pdf_qbin, scat.exp['rstep'], scat.get_r(), scat.exp['qmin'],
            torch.as_tensor(np.asarray(self.target_data, np.float64)),
            self.potential_name, want_grad=want_forces)
        e = out['energy'].cpu().numpy()[0]
        val, scale = float(e[0]), float(e[1])
        if self.potential_name == 'rw' and val == 1.0 and scale == 1.0:
            val, scale = 1, 1
        self.scale = scale
        self.results['energy'] = val * self.rw_to_eV
        if want_forces:
            g = out['grad'].double().cpu().numpy()
            k = -1.0 if self.true_forces else -0.5
            self.results['forces'] = k * self.rw_to_eV * g

    def calculate_energy(self, atoms):
        energy, scale = self.potential(self.exp_function(atoms),
                                       self.target_data)
        self.scale = scale
        self.results['energy'] = energy * self.rw_to_eV

    def calculate_forces(self, atoms):
        forces = self.grad(self.exp_grad_function(atoms),
                           self.exp_function(atoms),
                           self.target_data) * self.rw_to_eV
        if self.true_forces:
            forces = 2.0 * forces
        self.results['forces'] = forces

    def calculate_voxel_energy(self, atoms, resolution):
        pass

    def calculate_atomwise_energy(self, atoms):
        pass
