"""Oracle (test infrastructure only) for the single-atom Metropolis path.

Restates, in NumPy, what ``pyiid_mh_steps`` computes so the tests can check
it step by step:

* :func:`philox4x32_10` -- the counter-based generator of Salmon, Moraes,
  Dror and Shaw ("Parallel random numbers: as easy as 1, 2, 3", SC 2011),
  pinned by the published known-answer vectors in the tests.
* :func:`proposal` -- proposal ``t`` of chain ``c``: atom, displacement
  (Box-Muller in float32) and log u, from the generator words exactly as the
  device forms them.
* :func:`metropolis_accept` -- the acceptance rule of the reference's
  Monte Carlo moves: accept when ``u < exp(min(0, -beta dE))``
  (pyiid/sim/gcmc.py:13-114 add_atom / del_atom with mu = 0;
  pyiid/sim/hmc.py:66-92 mh_accept, whose ``temp`` argument multiplies the
  energy difference), i.e. ``log u < -conv (V' - V) / kT``.
* :func:`exact_delta_s` -- the change of the raw Debye sums when one atom
  moves, by full re-evaluation of both configurations in FP64 (the reference
  re-evaluates the whole configuration for every move).

Nothing here runs in the product path.
"""
import numpy as np

from . import debye_np

M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
W0, W1 = 0x9E3779B9, 0xBB67AE85
_MASK = np.uint64(0xFFFFFFFF)


def philox4x32_10(counter, key):
    """Philox4x32-10 of counters [..., 4] (uint32) under key (k0, k1).

    Round: (hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0) with (hi0, lo0) =
    M0 * c0 and (hi1, lo1) = M1 * c2; the key advances by the Weyl
    constants between rounds."""
    c = np.asarray(counter, dtype=np.uint64) & _MASK
    c0, c1, c2, c3 = c[..., 0], c[..., 1], c[..., 2], c[..., 3]
    k0, k1 = int(key[0]) & 0xFFFFFFFF, int(key[1]) & 0xFFFFFFFF
    for _ in range(10):
        p0 = M0 * c0
        p1 = M1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & _MASK
        hi1, lo1 = p1 >> np.uint64(32), p1 & _MASK
        c0, c1, c2, c3 = (hi1 ^ c1 ^ np.uint64(k0)), lo1, \
            (hi0 ^ c3 ^ np.uint64(k1)), lo0
        k0 = (k0 + W0) & 0xFFFFFFFF
        k1 = (k1 + W1) & 0xFFFFFFFF
    return np.stack([c0, c1, c2, c3], axis=-1).astype(np.uint32)


def _unit_float(x):
    """(2 * (x >> 9) + 1) * 2^-24 in float32: a float in (0, 1)."""
    x = np.asarray(x, dtype=np.uint64)
    return ((np.uint64(2) * (x >> np.uint64(9)) + np.uint64(1))
            .astype(np.float32) * np.float32(2.0 ** -24))


def proposal(seed, chain, step, n_atoms, sigma):
    """(atom, displacement float32 [3], log u) of proposal ``step`` of
    ``chain`` (counters (step lo, step hi, chain, 0/1), key = seed); log u
    is the float32 log of the float uniform of word 1 of the second block."""
    key = (seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF)
    slo, shi = step & 0xFFFFFFFF, (step >> 32) & 0xFFFFFFFF
    r0 = philox4x32_10([slo, shi, chain, 0], key)
    r1 = philox4x32_10([slo, shi, chain, 1], key)
    atom = (int(r0[0]) * int(n_atoms)) >> 32
    f32 = np.float32
    ra = np.sqrt(f32(-2.0) * np.log(_unit_float(r0[1])))
    ang = f32(2.0) * _unit_float(r0[2])
    rb = np.sqrt(f32(-2.0) * np.log(_unit_float(r0[3])))
    ang2 = f32(2.0) * _unit_float(r1[0])
    d = np.array([ra * np.cos(np.pi * np.float64(ang)),
                  ra * np.sin(np.pi * np.float64(ang)),
                  rb * np.cos(np.pi * np.float64(ang2))]) * np.float64(sigma)
    logu = float(np.log(_unit_float(r1[1])))
    return atom, d, logu


def metropolis_accept(logu, v_new, v_old, conv, kT):
    """log u < -conv (V' - V) / kT (False for NaN)."""
    with np.errstate(invalid='ignore'):
        return bool(logu < -conv * (v_new - v_old) / kT)


def raw_sums(positions, species, table, qbin):
    """S_k = sum_{a>b} f_a f_b sin(Q_k r)/r in FP64 (NaN where two atoms
    coincide), species-correct tables [S][K]."""
    x = np.asarray(positions, np.float64)
    n = len(x)
    k = table.shape[1]
    q = np.arange(k) * qbin
    s = np.zeros(k)
    if n < 2:
        return s
    ia, ib = np.triu_indices(n, 1)
    r = np.linalg.norm(x[ia] - x[ib], axis=1)
    f = table[species]
    for c0 in range(0, len(r), 20000):
        sl = slice(c0, c0 + 20000)
        with np.errstate(divide='ignore', invalid='ignore'):
            w = np.sin(np.outer(r[sl], q)) / r[sl, None]
        s += np.sum(f[ia[sl]].astype(np.float64) * f[ib[sl]] * w, axis=0)
    return s


def exact_delta_s(positions, species, table, qbin, atom, new_position):
    """S(x') - S(x) for moving ``atom`` to ``new_position`` (full
    re-evaluation of both configurations)."""
    x0 = np.asarray(positions, np.float64)
    x1 = x0.copy()
    x1[atom] = new_position
    return (raw_sums(x1, species, table, qbin) -
            raw_sums(x0, species, table, qbin))


def potential_of(positions, species, table, exp, gobs, kind='rw'):
    """Potential of one configuration on the PDF grid (FP64 oracle chain:
    F -> G -> Rw or chi^2) with species-correct tables [S][K]."""
    per_atom = np.asarray(table)[np.asarray(species)]
    return debye_np.potential_value(np.asarray(positions), per_atom, exp,
                                    np.asarray(gobs, np.float64), kind)
