"""No-U-Turn sampler over ASE-style Atoms (the reference's
``pyiid.sim.nuts_hmc.NUTSCanonicalEnsemble``, pyiid/sim/nuts_hmc.py:91-232).

One chain of :class:`pyiid_gb300.nuts.NUTSEngine` (Hoffman and Gelman's
efficient NUTS with dual averaging, grown leaf by leaf with keyed random
draws) driven by the calculator attached to the atoms: energies and forces
come from ``get_potential_energy`` / ``get_forces`` at every leapfrog point
and at the re-centred end point, as an ASE calculator recomputes them
when positions change.  The constructor arguments, ``step``/``run``, the
trajectory of accepted configurations, ``pe``, the observers and the
metadata counters keep the reference's meaning; the engine's module
docstring lists the conventions kept (post-exponential slice variable,
Emax = 200, escape depth, Maxwell-Boltzmann momenta, dual-averaging
constants).  A BatchedNUTS chain with the same seed and potential makes the
same decisions (the random draws are keyed by iteration and tree slot).
"""
from copy import deepcopy as dc
from time import time

import numpy as np
import torch

from ..nuts import NUTSEngine, Emax
from . import Ensemble

__all__ = ['NUTSCanonicalEnsemble', 'Emax']


class NUTSCanonicalEnsemble(Ensemble):
    """NUTS at a temperature (K), step size adapted by dual averaging."""

    def __init__(self, atoms, restart=None, logfile=None, trajectory=None,
                 temperature=100, escape_level=13, accept_target=.65,
                 momentum=None, seed=None, verbose=False):
        Ensemble.__init__(self, atoms, restart, logfile, trajectory, seed,
                          verbose)
        self.accept_target = accept_target
        self.temp = temperature
        self.escape_level = escape_level
        self.momentum = momentum
        self._work = dc(atoms)
        self._work.set_calculator(atoms.get_calculator())
        x0 = np.asarray(atoms.get_positions(), np.float64)[None]
        self._engine = NUTSEngine(
            self._evaluate, x0, atoms.get_masses(), temperature,
            [self.metadata['seed']], escape_level=escape_level,
            accept_target=accept_target, momentum=momentum,
            reevaluate_centred=True, dtype=torch.float64, device='cpu')
        self.metadata.update({'samples_total': 0, 'accepted_samples': 0})
        if verbose:
            print('initial step size', self.step_size)

    def _evaluate(self, x):
        a = self._work
        a.set_positions(x[0].numpy())
        u = float(a.get_potential_energy())
        f = np.asarray(a.get_forces(), np.float64)
        return (torch.tensor([u], dtype=torch.float64),
                torch.as_tensor(f)[None])

    @property
    def step_size(self):
        return float(self._engine.step[0])

    @property
    def mu(self):
        return float(self._engine.mu[0])

    def step(self):
        """One NUTS iteration; returns the configurations it accepted (or
        None), each appended to the trajectory with observers called."""
        e = self._engine
        n0 = len(e.samples[0])
        e.run(1)
        new = []
        for x in e.samples[0][n0:]:
            a = dc(self.traj[-1])
            a.set_calculator(self._work.get_calculator())
            a.set_positions(x.numpy())
            self.traj.append(a)
            new.append(a)
            a.get_forces()
            self.pe.append(a.get_potential_energy())
            self.call_observers()
        self.metadata['accepted_samples'] = int(e.accepted[0])
        self.metadata['samples_total'] = int(e.samples_total[0])
        self.metadata['leapfrog_steps'] = int(e.leapfrogs[0])
        if self.verbose:
            print('\tstep size', self.step_size, 'accepted', len(new))
        return new or None

    def estimate_simulation_duration(self, atoms, iterations):
        """Upper bound of the run time: every iteration at the escape depth
        (2^escape_level leapfrog steps of two force calls each)."""
        t0 = time()
        atoms.get_forces()
        tf = time() - t0
        t2 = time()
        atoms.get_potential_energy()
        te = time() - t2
        return iterations * (tf * 2 + te) * 2 ** self.escape_level
