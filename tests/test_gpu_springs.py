"""Spring potentials and MultiCalc on the GPU against the oracle
(oracle/springs_np.py), and grand-canonical Monte Carlo with springs as in
the reference's test_sim/test_gcmc.py."""
import numpy as np
import pytest

from oracle import springs_np as SP
from pyiid_gb300 import structures as S

pytestmark = pytest.mark.gpu

KWARGS = [{'k': 100, 'rt': 5., 'sp_type': 'rep'},
          {'k': 100, 'rt': 1., 'sp_type': 'com'},
          {'k': 100, 'rt': 1., 'sp_type': 'att'},
          {'k': 7.5, 'rt': 2.9, 'sp_type': 'rep'},
          {'k': 3.0, 'rt': 6.0, 'sp_type': 'att'}]


def cluster(n=150, seed=0):
    from pyiid_gb300.atoms import Atoms
    q = S.displaced(S.fcc_nearest(4.08, n), 0.3, seed)
    return Atoms(numbers=[79] * n, positions=q)


def relerr(a, b):
    return np.linalg.norm(np.asarray(a) - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize('kw', KWARGS)
def test_spring_matches_oracle(kw):
    from pyiid_gb300.calc.spring_calc import Spring
    atoms = cluster(seed=1)
    atoms.set_calculator(Spring(**kw))
    q = atoms.get_positions()
    com = atoms.get_center_of_mass()
    k, rt, t = kw['k'], kw['rt'], kw['sp_type']
    if t == 'com':
        e_ref = SP.com_spring_nrg(q, k, rt, com)
        f_ref = SP.com_spring_force(q, k, rt, com)
    elif t == 'att':
        e_ref, f_ref = SP.att_spring_nrg(q, k, rt), SP.att_spring_force(q, k, rt)
    else:
        e_ref, f_ref = SP.spring_nrg(q, k, rt), SP.spring_force(q, k, rt)
    e = atoms.get_potential_energy()
    assert abs(e - e_ref) <= 1e-6 * abs(e_ref) + 1e-9, (e, e_ref)
    f = atoms.get_forces()
    assert relerr(f, f_ref) < 1e-5, relerr(f, f_ref)
    aw = atoms.calc.calculate_atomwise_energy(atoms)
    aw_ref = SP.atomwise_nrg(q, k, rt, t, com)
    assert np.allclose(aw, aw_ref, rtol=1e-5,
                       atol=1e-6 * np.max(np.abs(aw_ref)))


@pytest.mark.parametrize('kw', KWARGS[:3])
def test_voxel_energy_matches_oracle(kw):
    from pyiid_gb300.calc.spring_calc import Spring
    atoms = cluster(40, seed=2)
    atoms.positions += 6.0
    atoms.set_cell(np.array([12., 12., 12.]))
    atoms.set_calculator(Spring(**kw))
    vox = atoms.calc.calculate_voxel_energy(atoms, 0.75)
    ref = SP.voxel_nrg(atoms.get_positions(), kw['k'], kw['rt'],
                       kw['sp_type'], np.diagonal(atoms.get_cell()), 0.75,
                       atoms.get_center_of_mass())
    assert vox.shape == ref.shape == (16, 16, 16)
    assert np.allclose(vox, ref, rtol=1e-5, atol=1e-6 * np.abs(ref).max())


def test_empty_and_single_atom():
    from pyiid_gb300.atoms import Atoms
    from pyiid_gb300.calc.spring_calc import Spring
    a = Atoms(numbers=[79], positions=[[0., 0., 0.]])
    a.set_calculator(Spring(k=10, rt=2.))
    assert a.get_potential_energy() == 0.0
    assert np.all(a.get_forces() == 0)


def test_multicalc_sums_its_calculators():
    from pyiid_gb300.calc.multi_calc import MultiCalc
    from pyiid_gb300.calc.spring_calc import Spring
    atoms = cluster(80, seed=3)
    calcs = [Spring(**KWARGS[0]), Spring(**KWARGS[2])]
    atoms.set_calculator(MultiCalc(calc_list=calcs))
    e = atoms.get_potential_energy()
    f = atoms.get_forces()
    q = atoms.get_positions()
    e_ref = SP.spring_nrg(q, 100, 5.) + SP.att_spring_nrg(q, 100, 1.)
    f_ref = SP.spring_force(q, 100, 5.) + SP.att_spring_force(q, 100, 1.)
    assert abs(e - e_ref) <= 1e-6 * e_ref
    assert relerr(f, f_ref) < 1e-5


def test_gcmc_with_springs_grows():
    """pyiid/tests/test_sim/test_gcmc.py: an atomic square with springs and
    a large chemical potential gains atoms."""
    from pyiid_gb300.atoms import Atoms
    from pyiid_gb300.calc.spring_calc import Spring
    from pyiid_gb300.sim.gcmc import GrandCanonicalEnsemble
    for resolution in (None, .1):
        atoms = Atoms(numbers=[79] * 4,
                      positions=[[0, 0, 0], [3, 0, 0], [0, 3, 0], [3, 3, 0]])
        atoms.set_cell(np.array([6., 6., 6.]))
        del atoms[-2:]
        n0 = len(atoms)
        atoms.set_calculator(Spring(k=10, rt=2.5))
        dyn = GrandCanonicalEnsemble(atoms, {'Au': 100.0}, temperature=1000,
                                     resolution=resolution, seed=1)
        traj, metadata = dyn.run(10)
        assert max(len(a) for a in traj) > n0
