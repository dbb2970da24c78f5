"""Samplers over ASE-style Atoms (pyiid/sim): leapfrog and the Ensemble base.

Same names and semantics as pyiid/sim/__init__.py:10-82; the forces and
energies come from whatever calculator is attached (for the scattering path,
Calc1D on the GB300 processor).  Batched, device-resident chains are in
:mod:`pyiid_gb300.sampling`.
"""
from copy import deepcopy as dc

import numpy as np
from numpy.random import RandomState

__all__ = ['leapfrog', 'Ensemble']


def leapfrog(atoms, step, center=True):
    """One velocity-Verlet step of size ``step`` on a copy of ``atoms``
    (pyiid/sim/__init__.py:10-38): half kick, drift, half kick."""
    latoms = dc(atoms)
    latoms.set_momenta(latoms.get_momenta() + 0.5 * step * latoms.get_forces())
    latoms.positions += step * latoms.get_velocities()
    latoms.set_momenta(latoms.get_momenta() + 0.5 * step * latoms.get_forces())
    if center:
        latoms.center()
    return latoms


class Ensemble(object):
    """Base of the Monte Carlo ensembles (pyiid/sim/__init__.py:41-82): keeps
    the trajectory, potential energies, metadata and observers."""

    def __init__(self, atoms, restart=None, logfile=None, trajectory=None,
                 seed=None, verbose=False):
        self.atoms = atoms
        self.restart = restart
        self.logfile = logfile
        self.trajectory = trajectory
        self.observers = []
        atoms.get_forces()
        atoms.get_potential_energy()
        if seed is None:
            seed = np.random.randint(0, 2 ** 31)
        self.verbose = verbose
        self.random_state = RandomState(seed)
        self.starting_atoms = dc(atoms)
        self.traj = [dc(atoms)]
        self.pe = []
        self.metadata = {'seed': seed}

    def attach(self, function, interval=1, *args, **kwargs):
        self.observers.append((function, interval, args, kwargs))

    def call_observers(self):
        n = len(self.traj)
        for function, interval, args, kwargs in self.observers:
            if interval > 0 and n % interval == 0:
                function(*args, **kwargs)

    def check_eq(self, eq_steps, tol):
        ret = np.cumsum(self.pe, dtype=float)
        ret[eq_steps:] = ret[eq_steps:] - ret[:-eq_steps]
        ret = ret[eq_steps - 1:] / eq_steps
        return np.sum(np.gradient(ret[eq_steps:])) < tol

    def run(self, steps=100000000, eq_steps=None, eq_tol=None, **kwargs):
        self.metadata['planned iterations'] = steps
        try:
            for i in range(steps):
                if eq_steps is not None:
                    if self.check_eq(eq_steps, eq_tol):
                        break
                if self.verbose:
                    print('iteration number', i)
                self.step()
        except KeyboardInterrupt:
            print('Interrupted, returning data')
        return self.traj, self.metadata

    def step(self):
        pass

    def estimate_simulation_duration(self, atoms, iterations):
        pass
