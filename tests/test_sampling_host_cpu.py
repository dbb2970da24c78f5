"""Host-side set-up of the batched samplers' potential (no device call):
grids, species packing of uneven configurations, tables, masses and the
argument checks of pyiid_gb300.sampling.PDFPotential."""
import numpy as np
import pytest

from oracle import debye_np as O
from pyiid_gb300.sampling import PDFPotential, experiment_grids
from pyiid_gb300.scatter_factors import atomic_mass, form_factor_array


@pytest.mark.parametrize('exp', [
    None,
    {'qmin': 0.6, 'qmax': 22.0, 'qbin': 0.13, 'rmin': 0.5, 'rmax': 12.0,
     'rstep': 0.05, 'sampling': 'full'},
    {'qmin': 1.1, 'qmax': 20.0, 'qbin': 0.1, 'rmin': 1.0, 'rmax': 15.0,
     'rstep': 0.02, 'sampling': 'ns'},
])
def test_grids_are_the_experiments(exp):
    e, qb, n_bins, r = experiment_grids(None if exp is None else dict(exp))
    want = O.update_experiment(None if exp is None else dict(exp))
    assert e == want
    assert qb == O.pdf_qbin(want)
    assert n_bins == len(O.scatter_vector(want, pdf=True))
    assert np.array_equal(r, O.r_grid(want))


def test_uneven_configurations_are_packed():
    numbers = [np.array([79, 79, 78]), np.array([78]), np.array([79, 46])]
    _, _, _, r = experiment_grids(None)
    pot = PDFPotential(numbers, np.zeros(len(r)), device='cpu')
    assert list(pot.offsets) == [0, 3, 4, 6]
    assert pot.n_configs == 3 and pot.n_total == 6
    assert list(pot.uniq) == [46, 78, 79]
    assert list(pot.species) == [2, 2, 1, 1, 2, 0]
    assert pot.table.shape == (3, pot.n_bins)
    q = np.arange(pot.n_bins) * pot.qstep
    assert np.allclose(pot.table[1], form_factor_array(78, q))
    assert np.allclose(pot.masses, [atomic_mass(z) for z in
                                    [79, 79, 78, 78, 79, 46]])
    assert list(pot.config_index().numpy()) == [0, 0, 0, 1, 2, 2]


def test_same_atoms_repeated_over_configurations():
    _, _, _, r = experiment_grids(None)
    pot = PDFPotential([79] * 5, np.zeros(len(r)), n_configs=4, device='cpu')
    assert list(pot.offsets) == [0, 5, 10, 15, 20]
    assert np.all(pot.species == 0) and pot.table.shape[0] == 1


def test_argument_checks():
    _, _, n_bins, r = experiment_grids(None)
    with pytest.raises(ValueError):
        PDFPotential([79] * 3, np.zeros(len(r) - 1), device='cpu')
    with pytest.raises(ValueError):
        PDFPotential([79, 78], np.zeros(len(r)), device='cpu',
                     table=np.ones((1, n_bins)))
    pot = PDFPotential([79, 78], np.zeros(len(r)), device='cpu',
                       table=np.ones((2, n_bins)))
    assert pot.table.dtype == np.float32
