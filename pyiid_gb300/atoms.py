"""A minimal ASE-compatible ``Atoms`` and ``Calculator`` (ASE is not installed).

Only what pyIID's scattering path and samplers use: positions, numbers,
per-atom arrays (copied on copy/slice/delete like ASE's), ``info``, momenta,
masses, velocities, the calculator protocol (``get_forces``,
``get_potential_energy``, ``get_total_energy``) and ``center``.  Units are
ASE's: Angstrom, eV, amu; time unit Angstrom * sqrt(amu / eV).
"""
import copy
import re

import numpy as np

from .scatter_factors import ELEMENTS, atomic_mass

__all__ = ['Atoms', 'Atom', 'Calculator', 'kB', 'fs',
           'MaxwellBoltzmannDistribution']

# CODATA 2018; ASE time unit = 1e10 * sqrt(e / amu) s^-1
_e = 1.602176634e-19
_amu = 1.66053906660e-27
_second = 1e10 * np.sqrt(_e / _amu)
fs = 1e-15 * _second
kB = 1.380649e-23 / _e  # eV / K

_SYM = {z: s for s, (z, _) in ELEMENTS.items()}


def _parse_formula(symbols):
    out = []
    for sym, cnt in re.findall(r'([A-Z][a-z]?)(\d*)', symbols):
        out += [ELEMENTS[sym][0]] * (int(cnt) if cnt else 1)
    return out


class Atom:
    """A view of one atom of an :class:`Atoms` (``atoms[i].position`` is
    writable, as in ASE) or a free atom to append."""

    def __init__(self, symbol='X', position=(0, 0, 0), atoms=None, index=None):
        self._atoms, self._index = atoms, index
        if atoms is None:
            self._number = ELEMENTS[symbol][0] if isinstance(symbol, str) \
                else int(symbol)
            self._position = np.array(position, dtype=np.float64)

    @property
    def number(self):
        if self._atoms is None:
            return self._number
        return int(self._atoms.numbers[self._index])

    @property
    def symbol(self):
        return _SYM[self.number]

    @property
    def position(self):
        if self._atoms is None:
            return self._position
        return self._atoms.arrays['positions'][self._index]

    @position.setter
    def position(self, value):
        self.position[:] = value


class Atoms:
    """ASE-like container of atoms (no cell / pbc semantics: free particles)."""

    def __init__(self, symbols=None, positions=None, numbers=None,
                 masses=None, momenta=None, calculator=None, info=None):
        if numbers is None:
            if symbols is None:
                numbers = []
            elif isinstance(symbols, str):
                numbers = _parse_formula(symbols)
            else:
                numbers = [ELEMENTS[s][0] if isinstance(s, str) else int(s)
                           for s in symbols]
        numbers = np.asarray(numbers, dtype=np.int64).reshape(-1)
        n = len(numbers)
        if positions is None:
            positions = np.zeros((n, 3))
        self.arrays = {
            'numbers': numbers.copy(),
            'positions': np.array(positions, dtype=np.float64).reshape(n, 3),
        }
        if masses is not None:
            self.arrays['masses'] = np.array(masses, dtype=np.float64)
        if momenta is not None:
            self.arrays['momenta'] = np.array(momenta, dtype=np.float64)
        self.info = dict(info or {})
        self.calc = calculator
        self.cell = np.zeros((3, 3))
        self.pbc = np.zeros(3, bool)

    # --------------------------------------------------------- arrays
    def __len__(self):
        return len(self.arrays['positions'])

    @property
    def numbers(self):
        return self.arrays['numbers']

    @numbers.setter
    def numbers(self, v):
        self.arrays['numbers'][:] = v

    @property
    def positions(self):
        return self.arrays['positions']

    @positions.setter
    def positions(self, v):
        self.arrays['positions'][:] = v

    def get_positions(self):
        return self.arrays['positions'].copy()

    def set_positions(self, newpositions):
        self.arrays['positions'][:] = newpositions

    def get_atomic_numbers(self):
        return self.arrays['numbers'].copy()

    def get_chemical_symbols(self):
        return [_SYM[int(z)] for z in self.numbers]

    def get_tags(self):
        return np.zeros(len(self), int)

    def set_array(self, name, a, dtype=None):
        if a is None:
            self.arrays.pop(name, None)
            return
        a = np.array(a, dtype=dtype)
        if len(a) != len(self):
            raise ValueError(f'array {name} has length {len(a)} != {len(self)}')
        self.arrays[name] = a

    def get_array(self, name, copy=True):
        return self.arrays[name].copy() if copy else self.arrays[name]

    def has(self, name):
        return name in self.arrays

    def get_masses(self):
        if 'masses' in self.arrays:
            return self.arrays['masses'].copy()
        return np.array([atomic_mass(z) for z in self.numbers])

    def set_masses(self, masses):
        self.set_array('masses', np.asarray(masses, dtype=np.float64))

    def get_momenta(self):
        if 'momenta' in self.arrays:
            return self.arrays['momenta'].copy()
        return np.zeros((len(self), 3))

    def set_momenta(self, momenta):
        self.set_array('momenta', np.asarray(momenta, dtype=np.float64))

    def get_velocities(self):
        return self.get_momenta() / self.get_masses()[:, None]

    def set_velocities(self, velocities):
        self.set_momenta(np.asarray(velocities) * self.get_masses()[:, None])

    def get_center_of_mass(self):
        m = self.get_masses()
        return (m[:, None] * self.positions).sum(0) / m.sum()

    def center(self, vacuum=None, axis=(0, 1, 2), about=None):
        """Translate so the bounding box is centred on ``about`` (default:
        the origin; there is no cell).  Energies are translation invariant."""
        if len(self) == 0:
            return
        p = self.positions
        target = np.zeros(3) if about is None else np.asarray(about, float)
        for i in np.atleast_1d(axis):
            p[:, i] += target[i] - 0.5 * (p[:, i].min() + p[:, i].max())

    # --------------------------------------------------- copy / indexing
    def copy(self):
        new = Atoms.__new__(Atoms)
        new.arrays = {k: v.copy() for k, v in self.arrays.items()}
        new.info = copy.deepcopy(self.info)
        new.calc = None
        new.cell = self.cell.copy()
        new.pbc = self.pbc.copy()
        return new

    def __deepcopy__(self, memo):
        new = self.copy()
        new.calc = copy.deepcopy(self.calc, memo) if self.calc is not None \
            else None
        return new

    def __getitem__(self, i):
        if isinstance(i, (int, np.integer)):
            n = len(self)
            if i < -n or i >= n:
                raise IndexError('atom index out of range')
            return Atom(atoms=self, index=int(i) % n)
        new = self.copy()
        idx = np.arange(len(self))[i]
        new.arrays = {k: v[idx].copy() for k, v in self.arrays.items()}
        return new

    def __delitem__(self, i):
        mask = np.ones(len(self), bool)
        mask[np.arange(len(self))[i]] = False
        self.arrays = {k: v[mask] for k, v in self.arrays.items()}

    def __add__(self, other):
        new = self.copy()
        new += other
        return new

    def __iadd__(self, other):
        if isinstance(other, Atom):
            other = Atoms(numbers=[other.number], positions=[other.position])
        n1, n2 = len(self), len(other)
        arrays = {}
        for k, v in self.arrays.items():
            if k in other.arrays:
                w = other.arrays[k]
            else:
                w = np.zeros((n2,) + v.shape[1:], v.dtype)
                if k == 'masses':
                    w = other.get_masses()
            arrays[k] = np.concatenate([v, w.astype(v.dtype)])
        for k, w in other.arrays.items():
            if k not in arrays:
                v = np.zeros((n1,) + w.shape[1:], w.dtype)
                if k == 'masses':
                    v = self.get_masses()
                arrays[k] = np.concatenate([v, w])
        self.arrays = arrays
        return self

    def append(self, atom):
        self += atom

    def get_cell(self):
        return self.cell.copy()

    def set_cell(self, cell):
        c = np.asarray(cell, dtype=float)
        self.cell = np.diag(c) if c.ndim == 1 else c.reshape(3, 3).copy()

    # --------------------------------------------------------- calculator
    def set_calculator(self, calc=None):
        self.calc = calc

    def get_calculator(self):
        return self.calc

    def _need_calc(self):
        if self.calc is None:
            raise RuntimeError('Atoms object has no calculator.')
        return self.calc

    def get_potential_energy(self):
        return self._need_calc().get_potential_energy(self)

    def get_forces(self):
        return self._need_calc().get_forces(self)

    def get_kinetic_energy(self):
        p = self.get_momenta()
        return 0.5 * float((p * p / self.get_masses()[:, None]).sum())

    def get_total_energy(self):
        return self.get_potential_energy() + self.get_kinetic_energy()

    def get_temperature(self):
        dof = 3 * len(self)
        return 2 * self.get_kinetic_energy() / (dof * kB) if dof else 0.0


def MaxwellBoltzmannDistribution(atoms, temp, force_temp=False, rng=None):
    """Maxwell-Boltzmann momenta at thermal energy ``temp`` (eV, i.e. kB*T),
    rescaled to exactly that kinetic temperature when ``force_temp``."""
    rng = np.random if rng is None else rng
    m = atoms.get_masses()[:, None]
    p = rng.normal(size=(len(atoms), 3)) * np.sqrt(m * temp)
    atoms.set_momenta(p)
    if force_temp and len(atoms):
        ke = atoms.get_kinetic_energy()
        cur = 2 * ke / (3 * len(atoms))
        if cur > 0:
            atoms.set_momenta(p * np.sqrt(temp / cur))


class Calculator:
    """ASE's calculator protocol: cached ``results`` invalidated when the
    atoms' positions or numbers change."""
    implemented_properties = []

    def __init__(self, restart=None, ignore_bad_restart_file=False,
                 label=None, atoms=None, **kwargs):
        self.results = {}
        self.atoms = None
        self.parameters = dict(kwargs)
        if atoms is not None:
            atoms.calc = self

    def check_state(self, atoms, tol=1e-15):
        if self.atoms is None:
            return ['positions', 'numbers']
        changes = []
        if (len(atoms) != len(self.atoms) or
                not np.allclose(atoms.positions, self.atoms.positions,
                                rtol=0, atol=tol)):
            changes.append('positions')
        if len(atoms) != len(self.atoms) or not np.array_equal(
                atoms.numbers, self.atoms.numbers):
            changes.append('numbers')
        return changes

    def calculate(self, atoms=None, properties=['energy'],
                  system_changes=['positions', 'numbers', 'cell', 'pbc',
                                  'charges', 'magmoms']):
        if atoms is not None:
            self.atoms = atoms.copy()

    def get_property(self, name, atoms=None, allow_calculation=True):
        if atoms is None:
            atoms = self.atoms
            system_changes = []
        else:
            system_changes = self.check_state(atoms)
            if system_changes:
                self.results = {}
        if name not in self.results:
            if not allow_calculation:
                return None
            self.calculate(atoms, [name], system_changes)
        result = self.results[name]
        return result.copy() if isinstance(result, np.ndarray) else result

    def get_potential_energy(self, atoms=None, force_consistent=False):
        return self.get_property('energy', atoms)

    def get_forces(self, atoms=None):
        return self.get_property('forces', atoms)

    def calculate_numerical_forces(self, atoms, d=0.001):
        """Central finite differences of the energy (ASE semantics)."""
        p0 = atoms.get_positions()
        f = np.zeros((len(atoms), 3))
        for a in range(len(atoms)):
            for i in range(3):
                atoms.positions[a, i] = p0[a, i] + d
                ep = self.get_potential_energy(atoms)
                atoms.positions[a, i] = p0[a, i] - d
                em = self.get_potential_energy(atoms)
                atoms.positions[a, i] = p0[a, i]
                f[a, i] = (em - ep) / (2 * d)
        return f
