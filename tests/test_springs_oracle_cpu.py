"""The spring oracle (oracle/springs_np.py) against the reference's own
spring tests (pyiid/tests/test_calc/test_spring*.py): the 4-atom squares of
setup_atomic_square, the three test parameter sets, energies >= 100,
torque-free forces, voxel energies equal to brute-force insertions and
atomwise energies equal to removals."""
import numpy as np
import pytest

from oracle import springs_np as SP

KWARGS = [{'k': 100, 'rt': 5., 'sp_type': 'rep'},
          {'k': 100, 'rt': 1., 'sp_type': 'com'},
          {'k': 100, 'rt': 1., 'sp_type': 'att'}]


def squares():
    q = np.array([[0, 0, 0], [3, 0, 0], [0, 3, 0], [3, 3, 0]], float)
    q -= 0.5 * (q.min(0) + q.max(0))
    return q, q * .75


def nrg(q, kw, com=None):
    if kw['sp_type'] == 'rep':
        return SP.spring_nrg(q, kw['k'], kw['rt'])
    if kw['sp_type'] == 'att':
        return SP.att_spring_nrg(q, kw['k'], kw['rt'])
    return SP.com_spring_nrg(q, kw['k'], kw['rt'],
                             np.mean(q, 0) if com is None else com)


def force(q, kw):
    if kw['sp_type'] == 'rep':
        return SP.spring_force(q, kw['k'], kw['rt'])
    if kw['sp_type'] == 'att':
        return SP.att_spring_force(q, kw['k'], kw['rt'])
    return SP.com_spring_force(q, kw['k'], kw['rt'], np.mean(q, 0))


@pytest.mark.parametrize('kw', KWARGS)
def test_known_squares(kw):
    q1, q2 = squares()
    assert nrg(q1, kw) >= 100
    f = force(q1, kw)
    com = q1.mean(0)
    for i in range(4):
        assert np.any(f[i])
        assert np.allclose(np.cross(q1[i] - com, f[i]), 0, atol=1e-5)


def test_known_values():
    q1, q2 = squares()
    # rep, rt = 5: 8 ordered sides at 3, 4 ordered diagonals at 3 sqrt 2
    d = np.float32(np.sqrt(np.float32(18)))
    want = 8 * 50 * (3 - 5.) ** 2 + 4 * 50 * (float(d) - 5.) ** 2
    assert abs(SP.spring_nrg(q1, 100, 5.) - want) < 1e-6 * want


@pytest.mark.parametrize('kw', [KWARGS[0], KWARGS[2]])
def test_voxel_energy_is_insertion_energy(kw):
    q1, _ = squares()
    q = q1 + 2.5  # inside a 7 A cell
    cell = np.array([7., 7., 7.])
    res = 1.
    vox = SP.voxel_nrg(q, kw['k'], kw['rt'], kw['sp_type'], cell, res)
    e0 = nrg(q, kw)
    brute = np.zeros(vox.shape)
    for i, j, k in np.ndindex(vox.shape):
        x = (np.array([i, j, k]) + .5) * res
        brute[i, j, k] = nrg(np.vstack([q, x]), kw) - e0
    assert np.allclose(vox, brute, rtol=1e-5, atol=1e-6 * np.abs(brute).max())


@pytest.mark.parametrize('kw', [KWARGS[0], KWARGS[2]])
def test_atomwise_energy_is_removal_energy(kw):
    q1, _ = squares()
    rng = np.random.default_rng(0)
    q = np.vstack([q1, rng.normal(0, 2, (6, 3))])
    aw = SP.atomwise_nrg(q, kw['k'], kw['rt'], kw['sp_type'])
    e0 = nrg(q, kw)
    brute = np.array([nrg(np.delete(q, i, 0), kw) - e0 for i in range(len(q))])
    assert np.allclose(aw, brute, rtol=1e-5, atol=1e-6 * np.abs(brute).max())
