"""Atomic form factors f(Q) and per-atom scatter tables.

The reference evaluates f(Q) with ``xraylib.FF_Rayl(Z, Q / 4 pi)``
(pyiid/experiments/elasticscatter/kernels/master_kernel.py:14-36).  xraylib is
not available here, so :func:`form_factor` is a labelled STAND-IN with the
right shape (f(0) = Z, smooth monotone decay): a three-Gaussian plus constant
form in s = sin(theta)/lambda = Q / (4 pi),

    f(Z, s) = Z * (0.45 e^{-b1 s^2} + 0.35 e^{-b2 s^2} + 0.15 e^{-b3 s^2} + 0.05),
    (b1, b2, b3) = (10, 2.5, 0.4) * (Z / 79)^0.25   [A^2].

Its values are not xraylib's.  Form factors are an INPUT of the scattering
kernels (a per-species table), so any table -- including a real one, such as
the reference's carbon table used in the tests -- can be passed instead.
"""
import math

import numpy as np

__all__ = ['form_factor', 'species_tables', 'ELEMENTS', 'atomic_number',
           'atomic_mass']

_A = (0.45, 0.35, 0.15)
_B = (10.0, 2.5, 0.4)
_C = 0.05

# symbol -> (Z, standard atomic weight in amu)
ELEMENTS = {
    'H': (1, 1.008), 'He': (2, 4.002602), 'C': (6, 12.011), 'N': (7, 14.007),
    'O': (8, 15.999), 'Al': (13, 26.9815385), 'Si': (14, 28.085),
    'Fe': (26, 55.845), 'Co': (27, 58.933194), 'Ni': (28, 58.6934),
    'Cu': (29, 63.546), 'Zn': (30, 65.38), 'Ag': (47, 107.8682),
    'Pd': (46, 106.42), 'Cd': (48, 112.414), 'Pt': (78, 195.084),
    'Au': (79, 196.966569), 'Pb': (82, 207.2),
}
_Z2SYM = {z: s for s, (z, _) in ELEMENTS.items()}


def atomic_number(symbol):
    return ELEMENTS[symbol][0]


def atomic_mass(z):
    return ELEMENTS[_Z2SYM[int(z)]][1]


def form_factor(z, s):
    """Stand-in f(Z, s) with s = Q / (4 pi) in 1/Angstrom (see module doc)."""
    scale = (float(z) / 79.0) ** 0.25
    s2 = float(s) * float(s)
    v = _C
    for a, b in zip(_A, _B):
        v += a * math.exp(-b * scale * s2)
    return float(z) * v


def form_factor_array(z, q):
    """Vectorised :func:`form_factor` over Q values (1/Angstrom)."""
    scale = (float(z) / 79.0) ** 0.25
    s2 = (np.asarray(q, dtype=np.float64) / (4 * np.pi)) ** 2
    v = np.full_like(s2, _C)
    for a, b in zip(_A, _B):
        v += a * np.exp(-b * scale * s2)
    return float(z) * v


def species_tables(numbers, qbin, n_bins, q_eval=None):
    """Species ids and a per-species table [S, n_bins] (float32).

    ``q_eval`` is the Q step at which f is evaluated (defaults to ``qbin``);
    the reference's PDF table uses the F(Q) step here
    (pyiid/experiments/elasticscatter/__init__.py:137).
    """
    numbers = np.asarray(numbers)
    uniq, species = np.unique(numbers, return_inverse=True)
    step = qbin if q_eval is None else q_eval
    q = np.arange(n_bins) * step
    tab = np.stack([form_factor_array(z, q) for z in uniq]).astype(np.float32)
    return species.astype(np.int32), tab, uniq
