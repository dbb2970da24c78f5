"""Spring potentials (pyiid/calc/spring_calc.py) on the GB300 library.

``Spring(k=10, rt=1.5, sp_type='rep'|'att'|'com')`` with the reference's
energies, forces (half of -dE/dq for the pair springs, as the reference's),
``calculate_voxel_energy`` and ``calculate_atomwise_energy``; the module
functions keep the reference's names and signatures.  Arithmetic runs in
``pyiid_spring`` / ``pyiid_spring_voxels`` (sm_103a).  Voxel grids take
int(cell diagonal / resolution) voxels per axis.
"""
import numpy as np

from ..atoms import Calculator

__all__ = ['Spring', 'spring_nrg', 'spring_force', 'voxel_spring_nrg',
           'atomwise_spring_nrg', 'com_spring_nrg', 'com_spring_force',
           'voxel_com_spring_nrg', 'atomwise_com_spring_nrg',
           'att_spring_nrg', 'att_spring_force', 'voxel_att_spring_nrg',
           'atomwise_att_spring_nrg']

_TYPES = {'rep': 0, 'att': 1, 'com': 2}


def _run(atoms, k, rt, sp_type, forces=False, atomwise=False):
    import ctypes
    import torch
    from .. import debye
    from .._native import context
    pos = debye.as_positions(np.asarray(atoms.get_positions(), np.float32))
    n = pos.shape[0]
    dev = pos.device
    com = None
    if sp_type == 'com':
        com = np.ascontiguousarray(atoms.get_center_of_mass(), np.float64)
    e = torch.empty(1, dtype=torch.float64, device=dev)
    f = torch.empty((n, 3), dtype=torch.float32, device=dev) if forces \
        else None
    aw = torch.empty(1 if sp_type == 'com' else max(n, 1),
                     dtype=torch.float64, device=dev) if atomwise else None
    context(dev.index).call(
        'pyiid_spring', ctypes.c_void_p(pos.data_ptr()), n, float(k),
        float(rt), _TYPES[sp_type],
        com.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        if com is not None else None,
        ctypes.c_void_p(e.data_ptr()),
        ctypes.c_void_p(f.data_ptr() if f is not None else 0),
        ctypes.c_void_p(aw.data_ptr() if aw is not None else 0))
    return e, f, aw


def _voxels(atoms, k, rt, sp_type, resolution):
    import ctypes
    import torch
    from .. import debye
    from .._native import context
    pos = debye.as_positions(np.asarray(atoms.get_positions(), np.float32))
    shape = tuple(int(c / resolution) for c in np.diagonal(atoms.get_cell()))
    out = torch.empty(shape, dtype=torch.float64, device=pos.device)
    com = np.ascontiguousarray(atoms.get_center_of_mass(), np.float64)
    context(pos.device.index).call(
        'pyiid_spring_voxels', ctypes.c_void_p(pos.data_ptr()), pos.shape[0],
        float(k), float(rt), _TYPES[sp_type],
        com.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), shape[0],
        shape[1], shape[2], float(resolution), ctypes.c_void_p(out.data_ptr()))
    return out.cpu().numpy()


def spring_nrg(atoms, k, rt):
    return float(_run(atoms, k, rt, 'rep')[0].item())


def spring_force(atoms, k, rt):
    return _run(atoms, k, rt, 'rep', forces=True)[1].double().cpu().numpy()


def voxel_spring_nrg(atoms, k_const, rt, resolution):
    return _voxels(atoms, k_const, rt, 'rep', resolution)


def atomwise_spring_nrg(atoms, k, rt):
    return _run(atoms, k, rt, 'rep', atomwise=True)[2].cpu().numpy()[
        :len(atoms)]


def com_spring_nrg(atoms, k, rt):
    return float(_run(atoms, k, rt, 'com')[0].item())


def com_spring_force(atoms, k, rt):
    return _run(atoms, k, rt, 'com', forces=True)[1].double().cpu().numpy()


def voxel_com_spring_nrg(atoms, k_const, rt, resolution):
    return _voxels(atoms, k_const, rt, 'com', resolution)


def atomwise_com_spring_nrg(atoms, k, rt):
    return float(_run(atoms, k, rt, 'com', atomwise=True)[2].item())


def att_spring_nrg(atoms, k, rt):
    return float(_run(atoms, k, rt, 'att')[0].item())


def att_spring_force(atoms, k, rt):
    return _run(atoms, k, rt, 'att', forces=True)[1].double().cpu().numpy()


def voxel_att_spring_nrg(atoms, k_const, rt, resolution):
    return _voxels(atoms, k_const, rt, 'att', resolution)


def atomwise_att_spring_nrg(atoms, k, rt):
    return _run(atoms, k, rt, 'att', atomwise=True)[2].cpu().numpy()[
        :len(atoms)]


class Spring(Calculator):
    """Spring Repulsion Potential Energy Surface (spring_calc.py:10-96)."""
    implemented_properties = ['energy', 'forces']

    def __init__(self, restart=None, ignore_bad_restart_file=False, label=None,
                 atoms=None, k=10, rt=1.5, sp_type='rep', **kwargs):
        Calculator.__init__(self, restart, ignore_bad_restart_file, label,
                            atoms, **kwargs)
        if sp_type not in _TYPES:
            raise NotImplementedError(f'spring type {sp_type!r}')
        self.sp_type = sp_type
        self.k = k
        self.rt = rt
        self.nrg_func = spring_nrg
        self.f_func = spring_force
        self.v_nrg = voxel_spring_nrg
        self.atomwise_nrg = atomwise_spring_nrg
        if sp_type == 'com':
            self.nrg_func = com_spring_nrg
            self.f_func = com_spring_force
            self.v_nrg = voxel_com_spring_nrg
            self.atomwise_nrg = atomwise_com_spring_nrg
        if sp_type == 'att':
            self.nrg_func = att_spring_nrg
            self.f_func = att_spring_force
            self.v_nrg = voxel_att_spring_nrg
            self.atomwise_nrg = atomwise_att_spring_nrg

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
        self.results['energy'] = self.nrg_func(atoms, self.k, self.rt)

    def calculate_forces(self, atoms):
        self.results['forces'] = self.f_func(atoms, self.k, self.rt)

    def calculate_voxel_energy(self, atoms, resolution):
        return self.v_nrg(atoms, self.k, self.rt, resolution)

    def calculate_atomwise_energy(self, atoms):
        return self.atomwise_nrg(atoms, self.k, self.rt)
