"""Fixed-trajectory HMC with adaptive step size (pyiid/sim/hmc.py).

The reference marks this module deprecated in favour of NUTS; it is kept for
API completeness with the same functions and conventions (velocities are
redrawn as N(0,1)/3/N, hmc.py:95-130; acceptance exp(diff * temp),
hmc.py:66-92).
"""
from copy import deepcopy as dc

import numpy as np

__all__ = ['leapfrog', 'simulate_dynamics', 'mh_accept', 'hmc_move',
           'run_hmc']


def leapfrog(atoms, step):
    """In-place kick-drift (hmc.py:10-30)."""
    f = atoms.get_forces()
    atoms.set_momenta(atoms.get_momenta() + step * f)
    atoms.set_positions(atoms.get_positions() + step * atoms.get_momenta())


def simulate_dynamics(atoms, stepsize, n_steps):
    """Half kick, n leapfrog steps, half kick (hmc.py:33-63)."""
    grad = atoms.get_forces()
    atoms.set_velocities(atoms.get_velocities() + 0.5 * stepsize * grad)
    atoms.set_positions(atoms.get_positions() +
                        stepsize * atoms.get_velocities())
    for _ in range(n_steps):
        leapfrog(atoms, stepsize)
    atoms.set_velocities(atoms.get_velocities() +
                         0.5 * stepsize * atoms.get_forces())


def mh_accept(initial_energy, next_energy, temp=1, rng=np.random):
    """Metropolis test on the Hamiltonian difference (hmc.py:66-92)."""
    with np.errstate(over='ignore'):
        canon_part_prob = np.exp((initial_energy - next_energy) * temp)
    return rng.random_sample((1,)) < canon_part_prob


def hmc_move(atoms, stepsize, n_steps, temp, rng=np.random):
    """One HMC proposal; returns (accepted, atoms to continue from)."""
    atoms.set_velocities(rng.normal(0, 1, (len(atoms), 3)) / 3 / len(atoms))
    prop = dc(atoms)
    simulate_dynamics(prop, stepsize, n_steps)
    accept = mh_accept(atoms.get_total_energy(), prop.get_total_energy(),
                       temp, rng)
    if accept:
        return True, prop
    return False, atoms


def run_hmc(atoms, iterations, stepsize, n_steps, avg_acceptance_slowness,
            avg_acceptance_rate, target_acceptance_rate, stepsize_inc,
            stepsize_dec, stepsize_min, stepsize_max, temp=1, wtraj=None,
            rng=np.random):
    """HMC with step size adapted to a target acceptance (hmc.py:133-209).
    Returns (traj, accept_list, accept_num)."""
    traj = [atoms]
    accept_list, accept_num = [], []
    i = 0
    try:
        while i < iterations:
            accept, atoms = hmc_move(atoms, stepsize, n_steps, temp, rng)
            if accept is True:
                traj += [atoms]
                accept_num.append(i)
                if wtraj is not None:
                    wtraj.write(atoms)
            accept_list.append(accept)
            avg_acceptance_rate = (avg_acceptance_slowness *
                                   avg_acceptance_rate +
                                   (1.0 - avg_acceptance_slowness) *
                                   np.average(np.array(accept_list)))
            if avg_acceptance_rate > target_acceptance_rate:
                stepsize *= stepsize_inc
            else:
                stepsize *= stepsize_dec
            stepsize = min(max(stepsize, stepsize_min), stepsize_max)
            i += 1
    except KeyboardInterrupt:
        pass
    return traj, accept_list, accept_num
