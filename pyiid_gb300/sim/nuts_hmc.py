"""No-U-Turn sampler with dual-averaging step size (pyiid/sim/nuts_hmc.py).

Same algorithm and conventions as the reference: slice variable in
post-exponential units (u in [0, 1] compared with exp(E0 - E)), the tree
built by recursive doubling with leapfrog steps, the U-turn criterion on the
span between the outermost states, the Emax = 200 slack, the emergency
escape depth, and the dual-averaging update of the step size
(nuts_hmc.py:160-232).  The temperature enters through the Maxwell-Boltzmann
momenta only, as in the reference (``beta`` is accepted but unused,
nuts_hmc.py:15-60).
"""
from copy import deepcopy as dc
from time import time

import numpy as np

from ..atoms import MaxwellBoltzmannDistribution, fs, kB
from . import Ensemble, leapfrog

__all__ = ['buildtree', 'NUTSCanonicalEnsemble', 'Emax']

Emax = 200


def buildtree(input_atoms, u, v, j, e, e0, rs, beta=1):
    """One subtree of depth j in direction v (nuts_hmc.py:15-88).  Returns
    (minus, plus, proposal, n, s, alpha_sum, n_alpha)."""
    if j == 0:
        atoms_prime = leapfrog(input_atoms, v * e)
        neg_delta_energy = e0 - atoms_prime.get_total_energy()
        with np.errstate(over='ignore'):
            exp1 = np.exp(neg_delta_energy)
            exp2 = np.exp(Emax + neg_delta_energy)
        n_prime = int(u <= exp1)
        s_prime = int(u < exp2)
        with np.errstate(over='ignore'):
            a = min(1, np.exp(-atoms_prime.get_total_energy() +
                              input_atoms.get_total_energy()))
        return atoms_prime, atoms_prime, atoms_prime, n_prime, s_prime, a, 1
    (neg_atoms, pos_atoms, atoms_prime, n_prime, s_prime, a_prime,
     na_prime) = buildtree(input_atoms, u, v, j - 1, e, e0, rs, beta)
    if s_prime == 1:
        if v == -1:
            (neg_atoms, _, atoms_pp, n_pp, s_pp, app, napp) = buildtree(
                neg_atoms, u, v, j - 1, e, e0, rs, beta)
        else:
            (_, pos_atoms, atoms_pp, n_pp, s_pp, app, napp) = buildtree(
                pos_atoms, u, v, j - 1, e, e0, rs, beta)
        if rs.uniform() < float(n_pp / (max(n_prime + n_pp, 1))):
            atoms_prime = atoms_pp
        a_prime = a_prime + app
        na_prime = na_prime + napp
        span = (pos_atoms.positions - neg_atoms.positions).flatten()
        s_prime = s_pp * (span.dot(neg_atoms.get_velocities().flatten()) >= 0
                          ) * (span.dot(pos_atoms.get_velocities().flatten()) >= 0)
        n_prime = n_prime + n_pp
    return (neg_atoms, pos_atoms, atoms_prime, n_prime, s_prime, a_prime,
            na_prime)


class NUTSCanonicalEnsemble(Ensemble):
    """NUTS at a temperature (K), step size adapted by dual averaging."""

    def __init__(self, atoms, restart=None, logfile=None, trajectory=None,
                 temperature=100, escape_level=13, accept_target=.65,
                 momentum=None, seed=None, verbose=False):
        Ensemble.__init__(self, atoms, restart, logfile, trajectory, seed,
                          verbose)
        self.accept_target = accept_target
        self.temp = temperature
        self.thermal_nrg = self.temp * kB
        self.momentum = momentum
        self.step_size = self._find_step_size(atoms, self.thermal_nrg)
        self.mu = np.log(10 * self.step_size)
        self.sim_hbar = 0
        self.gamma = 0.05
        self.t0 = 10
        self.metadata.update({'samples_total': 0, 'accepted_samples': 0})
        self.escape_level = escape_level
        self.m = 0

    def _mb(self, atoms, thermal_nrg):
        MaxwellBoltzmannDistribution(atoms, thermal_nrg, force_temp=True,
                                     rng=self.random_state)

    def _find_step_size(self, input_atoms, thermal_nrg=None, momentum=None):
        """Doubling / halving search for a reasonable first step size
        (nuts_hmc.py:116-158)."""
        atoms = dc(input_atoms)
        step_size = .5
        if thermal_nrg:
            self._mb(atoms, thermal_nrg)
        elif momentum:
            atoms.set_momenta(self.random_state.normal(0, 1, (len(atoms), 3)))
        atoms_prime = leapfrog(atoms, step_size)
        with np.errstate(over='ignore'):
            # a = +1 (grow) or -1 (shrink), kept a Python float so that the
            # threshold 2^-a is well defined for both signs
            a = 1.0 if np.exp(-1 * atoms_prime.get_total_energy() +
                              atoms.get_total_energy()) > 0.5 else -1.0
            while (np.exp(-1 * atoms_prime.get_total_energy() +
                          atoms.get_total_energy())) ** a > 2.0 ** -a:
                step_size *= 2 ** a
                if self.verbose:
                    print('trying step size', step_size)
                atoms_prime = leapfrog(atoms, step_size)
                if step_size < 1e-7 or step_size > 1e7:
                    step_size = 1.
                    break
        return step_size

    def step(self):
        new_configurations = []
        if self.verbose:
            print('\ttime step size', self.step_size / fs, 'fs')
        if self.momentum is None:
            self._mb(self.traj[-1], self.thermal_nrg)
        else:
            self.traj[-1].set_momenta(self.random_state.normal(
                0, 1, (len(self.traj[-1]), 3)))
        u = self.random_state.uniform(0, 1)
        e0 = self.traj[-1].get_total_energy()
        e = self.step_size
        n, s, j = 1, 1, 0
        neg_atoms = dc(self.traj[-1])
        pos_atoms = dc(self.traj[-1])
        a, na = 0.0, 1
        while s == 1:
            v = self.random_state.choice([-1, 1])
            if v == -1:
                (neg_atoms, _, atoms_prime, n_prime, s_prime, a, na) = \
                    buildtree(neg_atoms, u, v, j, e, e0, self.random_state,
                              1 / self.thermal_nrg)
            else:
                (_, pos_atoms, atoms_prime, n_prime, s_prime, a, na) = \
                    buildtree(pos_atoms, u, v, j, e, e0, self.random_state,
                              1 / self.thermal_nrg)
            if s_prime == 1 and self.random_state.uniform() < min(
                    1, n_prime * 1. / n):
                self.traj += [atoms_prime]
                self.metadata['accepted_samples'] += 1
                new_configurations.append(atoms_prime)
                atoms_prime.get_forces()
                self.pe.append(atoms_prime.get_potential_energy())
                self.call_observers()
            n = n + n_prime
            span = (pos_atoms.positions - neg_atoms.positions).flatten()
            s = s_prime * (span.dot(neg_atoms.get_velocities().flatten()) >= 0
                           ) * (span.dot(pos_atoms.get_velocities().flatten()) >= 0)
            j += 1
            self.metadata['samples_total'] += 2 ** j
            if j >= self.escape_level:
                s = 0
        w = 1. / (self.m + self.t0)
        self.sim_hbar = (1 - w) * self.sim_hbar + w * (self.accept_target -
                                                       a / na)
        self.step_size = np.exp(self.mu - (self.m ** .5 / self.gamma) *
                                self.sim_hbar)
        self.m += 1
        return new_configurations or None

    def estimate_simulation_duration(self, atoms, iterations):
        t0 = time()
        atoms.get_forces()
        tf = time() - t0
        t2 = time()
        atoms.get_potential_energy()
        te = time() - t2
        return iterations * (tf * 2 + te) * 2 ** self.escape_level
