"""The drop-in ElasticScatter's host logic on the CPU.

The processor plug-in contract (pyiid/experiments/elasticscatter/
__init__.py:206-292) is three callables; here they are test doubles backed
by the FP64 oracle, and the F -> G transform is the oracle's FFT form.  What
runs for real is the layer a pyIID user calls: the experiment grids, the
per-atom scatter tables cached on the Atoms object (with the reference's
quirks), the cache invalidation, the qmin slicing and zeroing of the
getters, and the S(Q) / I(Q) post-processing.  Everything is compared with
the reference's own recorded outputs at the reference tests' tolerances
(pyiid/tests/test_scatter.py:9-10).  tests/test_gpu_compat.py runs the same
getters on the GB300 processor.
"""
import numpy as np
import pytest

from oracle import debye_np as O
from pyiid_gb300.atoms import Atom, Atoms

RTOL, ATOL = 5e-4, 5e-5
EXPS = {
    'default': None,
    'short': {'qmin': 0.6, 'qmax': 22.0, 'qbin': 0.13, 'rmin': 0.5,
              'rmax': 12.0, 'rstep': 0.05, 'sampling': 'full'},
    'ns': {'qmin': 1.1, 'qmax': 20.0, 'qbin': 0.1, 'rmin': 1.0,
           'rmax': 15.0, 'rstep': 0.02, 'sampling': 'ns'},
}


@pytest.fixture
def ES(monkeypatch):
    """ElasticScatter with oracle-backed processor callables."""
    from pyiid_gb300.experiments import elasticscatter as es_mod

    def table(atoms, sum_type):
        return atoms.get_array('F(Q) scatter' if sum_type == 'fq'
                               else 'PDF scatter')

    def fq(atoms, qbin, sum_type='fq'):
        return O.fq(atoms.get_positions(), table(atoms, sum_type),
                    qbin).astype(np.float32)

    def grad(atoms, qbin, sum_type='fq'):
        return O.grad_fq(atoms.get_positions(), table(atoms, sum_type),
                         qbin).astype(np.float32)

    def set_processor(self, processor=None, kernel_type='flat'):
        self.fq, self.grad, self.grad_pdf = fq, grad, O.grad_pdf
        self.processor, self.alg = 'oracle stand-in', kernel_type
        return True

    monkeypatch.setattr(es_mod.ElasticScatter, 'set_processor', set_processor)
    monkeypatch.setattr(es_mod, 'get_pdf_at_qmin', O.pdf_fft)

    def make(exp_name, **kw):
        e = EXPS[exp_name]
        return es_mod.ElasticScatter(exp_dict=None if e is None else dict(e),
                                     **kw)
    return make


def close(a, b, rtol=RTOL, atol=ATOL):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    assert a.shape == b.shape
    np.testing.assert_allclose(np.nan_to_num(a), np.nan_to_num(b), rtol=rtol,
                               atol=atol)


@pytest.mark.parametrize('exp_name', ['default', 'short', 'ns'])
@pytest.mark.parametrize('tag', ['au2', 'square', 'rand20', 'alloy16'])
def test_getters_match_reference_outputs(golden, ES, tag, exp_name):
    key = f'{tag}__{exp_name}'
    s = ES(exp_name)
    atoms = Atoms(numbers=golden[key + '__numbers'],
                  positions=golden[key + '__positions'])
    fq = s.get_fq(atoms)
    close(fq, golden[key + '__fq'])
    # the per-atom tables are built once and cached on the Atoms object
    close(atoms.get_array('F(Q) scatter'), golden[key + '__fq_table'],
          rtol=1e-6, atol=0)
    close(atoms.get_array('PDF scatter'), golden[key + '__pdf_table'],
          rtol=1e-6, atol=0)
    fq2 = s.get_fq(atoms)
    assert fq is not fq2 and np.array_equal(fq, fq2)
    close(s.get_sq(atoms), golden[key + '__sq'])
    close(s.get_iq(atoms), golden[key + '__iq'], atol=5e-3)
    close(s.get_pdf(atoms), golden[key + '__pdf'])
    g = s.get_grad_fq(atoms)
    assert g.dtype == np.float32
    close(g, golden[key + '__grad_fq'])
    if key + '__grad_pdf' in golden.files:
        close(s.get_grad_pdf(atoms), golden[key + '__grad_pdf'])
    assert np.array_equal(s.get_r(), golden[key + '__r'])
    assert np.allclose(s.get_scatter_vector(), golden[key + '__q'])
    assert np.allclose(s.get_scatter_vector(pdf=True),
                       golden[key + '__q_pdf'])


def test_scatter_tables_are_rebuilt_when_the_atoms_change(golden, ES):
    """test_scatter_state.py: adding or deleting an atom, or changing the
    experiment, invalidates the cached tables."""
    key = 'rand20__default'
    s = ES('default')
    atoms = Atoms(numbers=golden[key + '__numbers'],
                  positions=golden[key + '__positions'])
    s.get_fq(atoms)
    assert atoms.get_array('F(Q) scatter').shape[0] == len(atoms)
    atoms.append(Atom('Au', [0.5, 0.5, 0.5]))
    fq = s.get_fq(atoms)
    assert atoms.get_array('F(Q) scatter').shape[0] == len(atoms)
    assert atoms.info['scatter_atoms'] == len(atoms)
    del atoms[0]
    fq2 = s.get_fq(atoms)
    assert atoms.get_array('F(Q) scatter').shape[0] == len(atoms)
    assert not np.array_equal(fq, fq2)
    s.update_experiment({'qmax': 20.0})
    s.get_fq(atoms)
    assert atoms.info['exp'] == s.exp
    assert atoms.get_array('F(Q) scatter').shape[1] == int(20.0 / 0.1)


def test_experiment_grids(ES):
    """update_experiment (__init__.py:180-204): the reference's defaults, the
    'ns' r step pi / qmax and the PDF Q step pi / (rmax + 12 pi / qmax)."""
    s = ES('default')
    assert s.exp == {'qmin': 0.0, 'qmax': 25, 'qbin': .1, 'rmin': 0.0,
                     'rmax': 40.0, 'rstep': .01, 'sampling': 'full'}
    assert abs(s.pdf_qbin - 0.0756865) < 1e-7
    assert len(s.get_r()) == 4000 and len(s.get_scatter_vector()) == 250
    s.update_experiment({'qmax': 20.0, 'sampling': 'ns'})
    assert abs(s.exp['rstep'] - np.pi / 20.0) < 1e-15
    assert abs(s.pdf_qbin - np.pi / (40.0 + 12 * np.pi / 20.0)) < 1e-15
    assert len(s.get_r()) == len(np.arange(0.0, 40.0, np.pi / 20.0))


@pytest.fixture
def oracle_potentials(monkeypatch):
    """The potential functions behind wrap_rw / wrap_grad_rw (and chi^2) as
    oracle doubles with the reference's signatures (master_kernel.py)."""
    import pyiid_gb300.calc as calc_mod

    def grad_rw(out, gpdf, gcalc, gobs, rw, scale):
        out[:] = O.get_grad_rw(gpdf, gcalc, gobs, rw, scale)

    def grad_chi(out, gpdf, gcalc, gobs, scale):
        out[:] = O.get_grad_chi_sq(gpdf, gcalc, gobs, scale)

    monkeypatch.setattr(calc_mod, 'get_rw',
                        lambda gobs, gcalc, weight=None: O.get_rw(gobs, gcalc))
    monkeypatch.setattr(calc_mod, 'get_chi_sq', O.get_chi_sq)
    monkeypatch.setattr(calc_mod, 'get_grad_rw', grad_rw)
    monkeypatch.setattr(calc_mod, 'get_grad_chi_sq', grad_chi)


def _pot_keys(g):
    return sorted({k.rsplit('__', 1)[0] for k in g.files
                   if k.startswith('pot')})


@pytest.mark.parametrize('idx', range(6))
def test_calc1d_energy_and_forces_follow_the_reference(golden, ES,
                                                       oracle_potentials,
                                                       idx):
    """Calc1D (pyiid/calc/calc_1d.py:9-95) on functions that are not the
    GB300 getters takes the reference's path: energy = conv * Rw (or chi^2)
    and forces = conv * the reference's gradient contraction (-1/2 of the
    true -dE/dx; twice that with true_forces)."""
    from pyiid_gb300.calc.calc_1d import Calc1D
    key = _pot_keys(golden)[idx]
    s = ES(key.split('__')[-1])
    target = golden[key + '__target']
    conv = 30.0
    for pot in ('rw', 'chi_sq'):
        for true_forces in (False, True):
            atoms = Atoms(numbers=golden[key + '__numbers'],
                          positions=golden[key + '__positions'])
            calc = Calc1D(target_data=target,
                          exp_function=lambda a: s.get_pdf(a),
                          exp_grad_function=lambda a: s.get_grad_pdf(a),
                          conv=conv, potential=pot, true_forces=true_forces)
            assert calc._fused is None
            atoms.set_calculator(calc)
            want_e = conv * float(golden[key + '__' + pot][0])
            e = atoms.get_potential_energy()
            assert abs(e - want_e) <= 1e-5 * max(1.0, abs(want_e)), (pot, e)
            want_f = conv * golden[key + '__grad_' + pot] * (
                2.0 if true_forces else 1.0)
            f = atoms.get_forces()
            err = np.linalg.norm(f - want_f) / max(np.linalg.norm(want_f),
                                                   1e-300)
            assert err <= 1e-4, (pot, true_forces, err)


@pytest.mark.parametrize('tag', ['au2', 'alloy16', 'rand20'])
def test_species_tables_reproduce_the_per_atom_arrays(golden, ES, tag):
    """The processor passes the kernels (species id per atom, one table row
    per species) instead of the reference's [N, K] per-atom arrays; the two
    must describe the same rows exactly, from the cached species column and
    from the fallback that derives it from the distinct rows."""
    from pyiid_gb300.experiments.elasticscatter.gb300_wrap import species_of
    key = f'{tag}__short'
    s = ES('short')
    atoms = Atoms(numbers=golden[key + '__numbers'],
                  positions=golden[key + '__positions'])
    s.get_fq(atoms)
    for sum_type, name in (('fq', 'F(Q) scatter'), ('PDF', 'PDF scatter')):
        per_atom = atoms.get_array(name).astype(np.float32)
        sp, tab = species_of(atoms, sum_type)
        assert sp.dtype == np.int32 and tab.dtype == np.float32
        assert np.array_equal(tab[sp], per_atom)
        saved = atoms.arrays.pop('GB300 species', None)
        try:
            sp2, tab2 = species_of(atoms, sum_type)
        finally:
            if saved is not None:
                atoms.arrays['GB300 species'] = saved
        assert np.array_equal(tab2[sp2], per_atom)
        assert len(tab2) == len(np.unique(per_atom, axis=0))


def test_species_column_is_not_trusted_after_an_edit(golden, ES):
    """An edited per-atom row (not the first or the last) makes the processor
    derive the species from the array itself instead of the cached column."""
    from pyiid_gb300.experiments.elasticscatter.gb300_wrap import species_of
    key = 'alloy16__short'
    s = ES('short')
    atoms = Atoms(numbers=golden[key + '__numbers'],
                  positions=golden[key + '__positions'])
    s.get_fq(atoms)
    arr = atoms.get_array('F(Q) scatter')    # a copy, as ASE returns
    arr[len(atoms) // 2] *= 1.5
    atoms.set_array('F(Q) scatter', arr)
    sp, tab = species_of(atoms, 'fq')
    assert np.array_equal(tab[sp], arr.astype(np.float32))


@pytest.mark.parametrize('exp_name', ['default', 'short'])
def test_noisy_getters_and_detector_map_match_reference(golden, ES, exp_name):
    """get_fq / get_pdf with an I(Q) standard deviation (scalar and per
    point) draw the same noise from the seeded ElasticScatter as the
    reference does (__init__.py:332-341, 376-383), and get_2d_scatter
    (__init__.py:448-475) maps the same pixels to the same bins, bin
    centres and bin edges included."""
    key = f'noise__alloy16__{exp_name}'
    s = ES(exp_name, seed=1234)
    base = 'alloy16__default'
    atoms = Atoms(numbers=golden[base + '__numbers'],
                  positions=golden[base + '__positions'])
    close(s.get_fq(atoms, iq_std=0.01), golden[key + '__fq_iq_std_scalar'])
    close(s.get_fq(atoms, iq_std=golden[key + '__iq_std_array']),
          golden[key + '__fq_iq_std_array'])
    close(s.get_pdf(atoms, iq_std=0.01), golden[key + '__pdf_iq_std_scalar'])
    n_qp = len(s.get_scatter_vector(pdf=True))
    close(s.get_pdf(atoms, iq_std=np.linspace(0.005, 0.02, n_qp)),
          golden[key + '__pdf_iq_std_array'])
    img = s.get_2d_scatter(atoms, golden[key + '__pixels'])
    ref = golden[key + '__2d']
    assert img.shape == ref.shape
    # the same pixels are lit (bin membership is exact) ...
    assert np.array_equal(img == 0, ref == 0)
    # ... with the same intensities
    close(img, ref)


def test_detector_map_is_the_bin_rule():
    """Pixel q lit by the bin Q_k with |q - Q_k| < qbin/2 (the later bin
    where two qualify, none at exact half-bin edges), NaN pixels dark."""
    from pyiid_gb300.experiments import elasticscatter as es_mod
    s = es_mod.ElasticScatter.__new__(es_mod.ElasticScatter)
    s.exp = {'qmin': 0.0, 'qmax': 1.0, 'qbin': 0.1}
    iq = np.arange(1.0, 11.0)
    s.get_iq = lambda atoms: iq
    q = s.exp['qbin'] * np.arange(10)
    s.get_scatter_vector = lambda pdf=False: q
    pix = np.array([[0.0, 0.04, 0.05, 0.06, 0.949, 0.95, 1.2, np.nan]])
    img = s.get_2d_scatter(None, pix)
    want = np.zeros(pix.size)
    for qk, ik in zip(q, iq):
        want[(qk - 0.05 < pix.ravel()) & (qk + 0.05 > pix.ravel())] = ik
    assert np.array_equal(img.ravel(), want)
