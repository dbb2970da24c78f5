"""Sum of several calculators (pyiid/calc/multi_calc.py:8-125).

Energies, forces, voxel and atomwise energies are the sums over
``calc_list``.  The reference evaluates each sub-calculator by attaching it
to the atoms (leaving the last one attached); this version asks each
sub-calculator directly and leaves the atoms' calculator unchanged.
"""
import numpy as np

from ..atoms import Calculator

__all__ = ['MultiCalc']


class MultiCalc(Calculator):
    """Composite potential energy surface: the sum of ``calc_list``."""
    implemented_properties = ['energy', 'forces']

    def __init__(self, restart=None, ignore_bad_restart_file=False, label=None,
                 atoms=None, calc_list=None, **kwargs):
        Calculator.__init__(self, restart, ignore_bad_restart_file, label,
                            atoms, **kwargs)
        self.calc_list = list(calc_list or [])

    def calculate(self, atoms=None, properties=['energy'],
                  system_changes=['positions', 'numbers', 'cell', 'pbc',
                                  'charges', 'magmoms']):
        Calculator.calculate(self, atoms, properties, system_changes)
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

    def calculate_energy(self, atoms):
        self.results['energy'] = sum(
            c.get_potential_energy(atoms) for c in self.calc_list)

    def calculate_forces(self, atoms):
        forces = np.zeros((len(atoms), 3))
        for c in self.calc_list:
            forces[:, :] += c.get_forces(atoms)
        self.results['forces'] = forces

    def calculate_voxel_energy(self, atoms, resolution):
        c = np.diagonal(atoms.get_cell())
        voxel_energy = np.zeros(tuple(int(x / resolution) for x in c))
        for calc in self.calc_list:
            try:
                voxel_energy += calc.calculate_voxel_energy(atoms, resolution)
            except AttributeError:
                pass
        return voxel_energy

    def calculate_atomwise_energy(self, atoms):
        nrg = np.zeros(len(atoms))
        for calc in self.calc_list:
            try:
                nrg += calc.calculate_atomwise_energy(atoms)
            except AttributeError:
                pass
        return nrg
