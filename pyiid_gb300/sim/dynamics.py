"""Classical dynamics (pyiid/sim/dynamics.py:5-28)."""
from . import leapfrog

__all__ = ['classical_dynamics']


def classical_dynamics(atoms, stepsize, n_steps):
    """Trajectory of ``n_steps`` leapfrog steps (list of Atoms, start first)."""
    atoms.get_forces()
    traj = [atoms]
    for _ in range(n_steps):
        traj.append(leapfrog(traj[-1], stepsize))
    return traj
