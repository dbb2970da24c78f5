"""Grand-canonical Monte Carlo (pyiid/sim/gcmc.py).

:func:`add_atom`, :func:`del_atom` and :class:`GrandCanonicalEnsemble` keep
the reference's interface, random-number use and acceptance rule
(pyiid/sim/gcmc.py:13-114, 117-184):

* a step removes an atom when ``random_state.uniform() >= .5``, else adds one;
* addition: element ``np.random.choice`` of the chemical potentials' keys,
  position ``np.random.uniform(0, max(cell, axis 0))`` (or a random voxel of
  size ``resolution`` plus ``random_state.uniform``), accepted when
  ``np.random.random() < exp(min(0, -beta dE + beta mu))``;
* removal (only when more than one atom is left): index
  ``random_state.choice``, accepted when
  ``np.random.random() < exp(min(0, -beta dE - beta mu))`` and dE is not NaN.

The reference evaluates the energy of the whole trial configuration for
every move.  When the atoms carry a :class:`pyiid_gb300.calc.Calc1D` on the
GB300 ElasticScatter (PDF potential) and hold a single element that is also
the only chemical-potential key, :class:`GrandCanonicalEnsemble` obtains the
same energy differences in O(N K) on the device instead (``pyiid_mc_propose``
/ ``pyiid_mc_accept``): the same proposals, the same decisions, the same
trajectory.  Other systems use the reference algorithm with the attached
calculator.  (The reference's ``del_atom`` prints the atom count on every
call; that print is not reproduced.)
"""
from copy import deepcopy as dc

import numpy as np

from ..atoms import Atom, kB
from . import Ensemble

__all__ = ['add_atom', 'del_atom', 'GrandCanonicalEnsemble']

# ElasticScatter's per-atom caches on Atoms (rebuilt on demand whenever the
# atom count differs from info['scatter_atoms'])
_SCATTER_CACHE = ('F(Q) scatter', 'PDF scatter', 'GB300 species')


def _copy_without_scatter_cache(atoms):
    """atoms.copy() without the scatter caches: the O(N K) engine never
    reads them, an insertion or removal invalidates them anyway, and at a
    few hundred atoms copying them dominates the cost of a move."""
    saved = {k: atoms.arrays.pop(k) for k in _SCATTER_CACHE
             if k in atoms.arrays}
    try:
        return atoms.copy()
    finally:
        atoms.arrays.update(saved)


def _insertion_position(atoms, random_state, resolution):
    """New-atom position as pyiid/sim/gcmc.py:44-51 draws it."""
    if resolution is None:
        return np.random.uniform(0, np.max(atoms.get_cell(), 0))
    c = np.int32(np.ceil(np.diagonal(atoms.get_cell()) / resolution))
    qvr = np.random.choice(int(np.prod(c)))
    qv = np.asarray(np.unravel_index(qvr, c))
    return (qv + random_state.uniform(0, 1, 3)) * resolution


def add_atom(atoms, chem_potentials, beta, random_state, resolution=None):
    """Trial insertion (pyiid/sim/gcmc.py:13-65): the new configuration if
    accepted, else None."""
    atoms_prime = dc(atoms)
    new_symbol = np.random.choice(list(chem_potentials.keys()))
    e0 = atoms.get_potential_energy()
    new_position = _insertion_position(atoms, random_state, resolution)
    atoms_prime.append(Atom(new_symbol, np.asarray(new_position)))
    delta_energy = atoms_prime.get_potential_energy() - e0
    mu = chem_potentials[new_symbol]
    with np.errstate(invalid='ignore', over='ignore'):
        if np.random.random() < np.exp(
                min([0, -1. * beta * delta_energy + beta * mu])):
            return atoms_prime
    return None


def del_atom(atoms, chem_potentials, beta, random_state):
    """Trial removal (pyiid/sim/gcmc.py:68-114): the new configuration if
    accepted, else None."""
    if len(atoms) <= 1:
        return None
    atoms_prime = dc(atoms)
    e0 = atoms.get_potential_energy()
    del_atom_index = random_state.choice(range(len(atoms)))
    del_symbol = atoms_prime[del_atom_index].symbol
    del atoms_prime[del_atom_index]
    delta_energy = atoms_prime.get_potential_energy() - e0
    mu = chem_potentials[del_symbol]
    with np.errstate(invalid='ignore', over='ignore'):
        if np.random.random() < np.exp(
                min([0, -1. * beta * delta_energy - beta * mu])) and \
                not np.isnan(delta_energy):
            return atoms_prime
    return None


class _IncrementalPDF:
    """Single-configuration state of the O(N K) engine: positions on the
    device, the running Debye sums and Gram scalars, the current energy."""

    def __init__(self, atoms, calc):
        import torch
        from .. import debye
        from ..experiments.elasticscatter.gb300_wrap import species_of
        scat = calc._fused
        scat._ensure(atoms)
        sp, tab = species_of(atoms, 'PDF')
        self.tab = np.ascontiguousarray(tab[:1], np.float32)
        self.qstep = scat.pdf_qbin
        self.rstep = scat.exp['rstep']
        self.rgrid = np.asarray(scat.get_r(), np.float64)
        self.qmin = scat.exp['qmin']
        self.kind = calc.potential_name
        self.conv = calc.rw_to_eV
        self.gobs = torch.as_tensor(np.asarray(calc.target_data, np.float64),
                                    device='cuda')
        self.x = torch.as_tensor(np.asarray(atoms.get_positions(), np.float32),
                                 device='cuda').contiguous()
        self._debye = debye
        self._init()

    def _args(self):
        n = self.x.shape[0]
        return (self.x, np.zeros(n, np.int32), np.array([0, n]), self.tab,
                self.qstep, self.rstep, self.rgrid, self.qmin)

    def _init(self):
        self.state = self._debye.mh_init(*self._args(), self.gobs,
                                         kind=self.kind)
        self.energy = self._value(self.state['energy'][0, 0].item())

    def _value(self, v):
        if self.kind == 'rw' and v == 1.0:
            v = 1
        return v * self.conv

    def propose(self, mode, atom=0, xyz=(0., 0., 0.)):
        """Energy of the trial configuration (state unchanged)."""
        ev = self._debye.mc_propose(*self._args(), self.state, [mode], [atom],
                                    np.asarray(xyz, np.float32).reshape(1, 3),
                                    [0], kind=self.kind)
        return self._value(ev[0, 0].item())

    def accept(self, mode, atom=0, xyz=(0., 0., 0.)):
        import torch
        self._debye.mc_accept(self.state, [True])
        if mode == self._debye.MOVE_INSERT:
            new = torch.as_tensor(np.asarray(xyz, np.float32).reshape(1, 3),
                                  device='cuda')
            self.x = torch.cat([self.x, new]).contiguous()
        elif mode == self._debye.MOVE_REMOVE:
            a = int(atom)
            self.x = torch.cat([self.x[:a], self.x[a + 1:]]).contiguous()
        else:
            self.x[atom] = torch.as_tensor(np.asarray(xyz, np.float32),
                                           device='cuda')
        self.energy = self._value(self.state['energy'][0, 0].item())


def _incremental_engine(atoms, chem_potentials):
    """The O(N K) engine when the system qualifies, else None."""
    from ..calc.calc_1d import Calc1D
    calc = atoms.get_calculator()
    if not isinstance(calc, Calc1D) or calc._fused is None:
        return None
    z = np.unique(atoms.get_atomic_numbers())
    if len(z) != 1 or len(atoms) < 1:
        return None
    sym = atoms[0].symbol
    if list(chem_potentials.keys()) != [sym]:
        return None
    try:
        return _IncrementalPDF(atoms, calc)
    except Exception:  # noqa: BLE001 -- e.g. a grid above the engine's limits
        return None


class GrandCanonicalEnsemble(Ensemble):
    """Grand Canonical Monte Carlo simulation (pyiid/sim/gcmc.py:117-184).

    ``incremental``: None (default) uses the O(N K) device engine when the
    system qualifies (see the module docstring), False never."""

    def __init__(self, atoms, chemical_potentials, temperature=100,
                 restart=None, logfile=None, trajectory=None, seed=None,
                 verbose=False, resolution=None, incremental=None):
        Ensemble.__init__(self, atoms, restart, logfile, trajectory, seed,
                          verbose)
        self.beta = 1. / (temperature * kB)
        self.chem_pot = chemical_potentials
        self.metadata = {'rejected_additions': 0, 'accepted_removals': 0,
                         'accepted_additions': 0, 'rejected_removals': 0}
        self.resolution = resolution
        self._engine = None
        if incremental is None or incremental:
            self._engine = _incremental_engine(self.traj[-1],
                                               chemical_potentials)

    # ------------------------------------------------ O(N K) engine moves
    def _fast_add(self, atoms):
        from ..debye import MOVE_INSERT
        eng = self._engine
        new_symbol = np.random.choice(list(self.chem_pot.keys()))
        e0 = eng.energy
        new_position = _insertion_position(atoms, self.random_state,
                                           self.resolution)
        e1 = eng.propose(MOVE_INSERT, 0, new_position)
        delta_energy = e1 - e0
        mu = self.chem_pot[new_symbol]
        with np.errstate(invalid='ignore', over='ignore'):
            ok = np.random.random() < np.exp(
                min([0, -1. * self.beta * delta_energy + self.beta * mu]))
        if not ok:
            return None
        eng.accept(MOVE_INSERT, 0, new_position)
        atoms_prime = _copy_without_scatter_cache(atoms)
        atoms_prime.append(Atom(new_symbol, np.asarray(new_position)))
        return self._attach(atoms_prime, atoms)

    def _fast_del(self, atoms):
        from ..debye import MOVE_REMOVE
        eng = self._engine
        if len(atoms) <= 1:
            return None
        e0 = eng.energy
        idx = int(self.random_state.choice(range(len(atoms))))
        del_symbol = atoms[idx].symbol
        e1 = eng.propose(MOVE_REMOVE, idx)
        delta_energy = e1 - e0
        mu = self.chem_pot[del_symbol]
        with np.errstate(invalid='ignore', over='ignore'):
            ok = np.random.random() < np.exp(
                min([0, -1. * self.beta * delta_energy - self.beta * mu])) \
                and not np.isnan(delta_energy)
        if not ok:
            return None
        eng.accept(MOVE_REMOVE, idx)
        atoms_prime = _copy_without_scatter_cache(atoms)
        del atoms_prime[idx]
        return self._attach(atoms_prime, atoms)

    def _attach(self, atoms_prime, atoms):
        """Share the calculator; its cached energy is the engine's."""
        calc = atoms.get_calculator()
        atoms_prime.set_calculator(calc)
        calc.atoms = atoms_prime.copy()
        calc.results = {'energy': self._engine.energy}
        return atoms_prime

    def step(self):
        if self.random_state.uniform() >= .5:
            mv = 'remove'
            if self._engine is not None:
                new_atoms = self._fast_del(self.traj[-1])
            else:
                new_atoms = del_atom(self.traj[-1], self.chem_pot, self.beta,
                                     self.random_state)
        else:
            mv = 'add'
            if self._engine is not None:
                new_atoms = self._fast_add(self.traj[-1])
            else:
                new_atoms = add_atom(self.traj[-1], self.chem_pot, self.beta,
                                     self.random_state,
                                     resolution=self.resolution)
        if new_atoms is not None:
            if self.verbose:
                print('\t' + mv + ' atom accepted', len(new_atoms))
            if mv == 'add':
                self.metadata['accepted_additions'] += 1
            else:
                self.metadata['accepted_removals'] += 1
            self.traj.append(new_atoms)
            return [new_atoms]
        if self.verbose:
            print('\t' + mv + ' atom rejected', len(self.traj[-1]))
        if mv == 'add':
            self.metadata['rejected_additions'] += 1
        else:
            self.metadata['rejected_removals'] += 1
        return None

    def estimate_simulation_duration(self, atoms, iterations):
        from time import time
        t2 = time()
        atoms.get_potential_energy()
        te = time() - t2
        return te * iterations
