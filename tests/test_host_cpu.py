"""Host-side logic that needs no GPU: the Atoms shim, units, structures,
form factors, processor selection without a device."""
import numpy as np
import pytest

from conftest import gpu_available
from pyiid_gb300 import structures as S
from pyiid_gb300.atoms import (Atoms, Atom, Calculator, kB, fs,
                               MaxwellBoltzmannDistribution)
from pyiid_gb300.scatter_factors import (form_factor, form_factor_array,
                                         species_tables)


def test_units():
    assert abs(kB - 8.617333262e-05) < 1e-12
    assert abs(fs - 0.09822694788464063) < 1e-9


def test_atoms_basics():
    a = Atoms('Au4', [[0, 0, 0], [3, 0, 0], [0, 3, 0], [3, 3, 0]])
    assert len(a) == 4 and list(a.numbers) == [79] * 4
    assert a.get_chemical_symbols() == ['Au'] * 4
    a.positions *= .75
    assert np.allclose(a.positions[1], [2.25, 0, 0])
    a[1].position[0] += 1
    assert np.isclose(a.positions[1, 0], 3.25)
    b = a + Atom('Pt', [1, 1, 1])
    assert len(b) == 5 and b.numbers[-1] == 78
    a.set_array('x', np.arange(4))
    c = a.copy()
    del c[0]
    assert len(c) == 3 and list(c.get_array('x')) == [1, 2, 3]
    assert list(a.get_array('x')) == [0, 1, 2, 3]
    a.center()
    p = a.positions
    assert np.allclose(0.5 * (p.min(0) + p.max(0)), 0)


def test_maxwell_boltzmann_force_temp():
    a = Atoms('Au50', np.random.default_rng(0).random((50, 3)) * 10)
    MaxwellBoltzmannDistribution(a, 300 * kB, force_temp=True,
                                 rng=np.random.default_rng(1))
    assert abs(a.get_temperature() - 300) < 1e-6
    assert np.allclose(a.get_velocities() * a.get_masses()[:, None],
                       a.get_momenta())


class _Quad(Calculator):
    implemented_properties = ['energy', 'forces']

    def calculate(self, atoms=None, properties=['energy'], system_changes=()):
        Calculator.calculate(self, atoms, properties, system_changes)
        x = self.atoms.positions
        self.results['energy'] = float((x ** 2).sum())
        self.results['forces'] = -2 * x


def test_calculator_protocol_and_numerical_forces():
    a = Atoms('Au3', [[0, 0, 1], [1, 0, 0], [0, 2, 0]])
    a.set_calculator(_Quad())
    assert a.get_potential_energy() == 6.0
    f = a.get_forces()
    assert np.allclose(f, -2 * a.positions)
    assert np.allclose(a.calc.calculate_numerical_forces(a, d=1e-4), f,
                       atol=1e-6)
    a.positions[0, 0] = 1.0
    assert a.get_potential_energy() == 7.0   # cache invalidated


def test_fcc_structures_match_workload_facts():
    assert len(S.fcc_sphere(4.08, 10.0)) == 249
    p = S.fcc_nearest(3.92, 20000)
    assert p.shape == (20000, 3)
    assert abs(np.sqrt((p ** 2).sum(1)).max() - 41.578) < 1e-2
    q = S.fcc_nearest(4.0, 2000)
    assert abs(np.sqrt((q ** 2).sum(1)).max() - 19.799) < 1e-2
    d = S.displaced(p[:10], 0.02, 2)
    assert d.dtype == np.float32
    assert np.array_equal(d, S.displaced(p[:10], 0.02, 2))


def test_form_factor_shape():
    assert abs(form_factor(79, 0.0) - 79) < 1e-12
    f = form_factor_array(79, np.arange(0, 30, 0.1))
    assert np.all(np.diff(f) < 0) and f[-1] > 0
    sp, tab, uniq = species_tables([79, 78, 79, 6], 0.1, 100)
    assert list(uniq) == [6, 78, 79] and list(sp) == [2, 1, 2, 0]
    assert tab.shape == (3, 100) and tab.dtype == np.float32


@pytest.mark.skipif(gpu_available(), reason='checks the no-GPU behaviour')
def test_no_cpu_fallback_without_gpu():
    from pyiid_gb300.experiments.elasticscatter import ElasticScatter
    with pytest.raises(RuntimeError, match='no CPU fallback'):
        ElasticScatter()
    from pyiid_gb300 import debye
    from pyiid_gb300._native import NativeError
    with pytest.raises(NativeError):
        debye.fq(np.zeros((2, 3), np.float32), np.zeros(2, np.int32),
                 np.ones((1, 10), np.float32), 0.1)


def test_atoms_formulas_indexing_and_arrays():
    """ASE semantics a drop-in user relies on: formulas, atom views that
    write through, slices and boolean masks as new Atoms, deletion keeping
    every per-atom array aligned, concatenation filling missing arrays."""
    a = Atoms('Au2PtPd', [[0, 0, 0], [1, 0, 0], [2, 0, 0], [3, 0, 0]])
    assert list(a.numbers) == [79, 79, 78, 46]
    a.set_array('tag', np.arange(4) * 10)
    a.set_momenta(np.arange(12.0).reshape(4, 3))
    a[2].position = [5.0, 5.0, 5.0]                 # view writes through
    assert np.array_equal(a.positions[2], [5, 5, 5])
    assert a[-1].symbol == 'Pd'
    with pytest.raises(IndexError):
        a[4]
    b = a[1:3]
    assert len(b) == 2 and list(b.get_array('tag')) == [10, 20]
    c = a[a.numbers == 79]
    assert list(c.numbers) == [79, 79]
    del a[[0, 2]]
    assert list(a.numbers) == [79, 46]
    assert list(a.get_array('tag')) == [10, 30]
    assert np.array_equal(a.get_momenta()[1], [9, 10, 11])
    d = a + Atoms('Pt', [[7, 7, 7]])
    assert list(d.numbers) == [79, 46, 78]
    assert d.get_array('tag')[-1] == 0 and np.all(d.get_momenta()[-1] == 0)
    with pytest.raises(ValueError):
        d.set_array('tag', np.arange(5))
    d.set_array('tag', None)
    assert not d.has('tag')
    # get_array copies unless asked not to
    arr = d.get_array('numbers')
    arr[0] = 1
    assert d.numbers[0] == 79
    d.get_array('numbers', copy=False)[0] = 1
    assert d.numbers[0] == 1


def test_atoms_mechanics():
    a = Atoms('H2Au', [[0, 0, 0], [2, 0, 0], [0, 0, 4]])
    m = a.get_masses()
    com = (m[:, None] * a.positions).sum(0) / m.sum()
    assert np.allclose(a.get_center_of_mass(), com)
    a.set_velocities(np.ones((3, 3)))
    assert np.allclose(a.get_momenta(), m[:, None])
    ke = 0.5 * 3 * m.sum()
    assert abs(a.get_kinetic_energy() - ke) < 1e-12
    assert abs(a.get_temperature() - 2 * ke / (9 * kB)) < 1e-9
    a.center(about=[1.0, 1.0, 1.0])
    p = a.positions
    assert np.allclose(0.5 * (p.min(0) + p.max(0)), [1, 1, 1])
    e = Atoms()
    assert len(e) == 0 and e.get_temperature() == 0.0
