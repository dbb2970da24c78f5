"""Batched NUTS on the GPU: every chain of a BatchedNUTS batch (the tree
grown on the device for all chains in lock step) reproduces a sequential
NUTSCanonicalEnsemble run on a Calc1D of the same potential (pyiid/sim/
nuts_hmc.py's sampler through the drop-in calculator) with the same seed,
sample for sample."""
import numpy as np
import pytest

from pyiid_gb300 import structures as S

pytestmark = pytest.mark.gpu

EXP = {'qmin': 0.6, 'qmax': 18.0, 'rmax': 10.0, 'rstep': 0.04}


def setup(n=22, chains=3):
    from pyiid_gb300.atoms import Atoms
    from pyiid_gb300.calc.calc_1d import Calc1D
    from pyiid_gb300.experiments.elasticscatter import ElasticScatter
    from pyiid_gb300.experiments.elasticscatter.gb300_wrap import species_of
    s = ElasticScatter(exp_dict=dict(EXP))
    ref = Atoms(numbers=[79] * n, positions=S.fcc_nearest(4.08, n))
    target = s.get_pdf(ref)
    starts = [S.displaced(S.fcc_nearest(4.08, n), 0.08, 10 + c)
              for c in range(chains)]
    probe = Atoms(numbers=[79] * n, positions=starts[0])
    s._ensure(probe)
    _, tab = species_of(probe, 'PDF')

    def calc():
        return Calc1D(target_data=target, exp_function=s.get_pdf,
                      exp_grad_function=s.get_grad_pdf, conv=50.)
    return s, target, starts, tab, calc


def test_batched_chains_reproduce_sequential_nuts():
    from pyiid_gb300.atoms import Atoms
    from pyiid_gb300.nuts import BatchedNUTS
    from pyiid_gb300.sampling import PDFPotential
    from pyiid_gb300.sim.nuts_hmc import NUTSCanonicalEnsemble
    s, target, starts, tab, calc = setup()
    seeds = [3, 17, 29]
    iters = 3
    pot = PDFPotential([79] * len(starts[0]), target, dict(EXP), conv=50.,
                       n_configs=len(starts), table=tab)
    bn = BatchedNUTS(pot, np.stack(starts), temperature=300, seeds=seeds,
                     escape_level=6)
    bn.step(iters)
    for c, seed in enumerate(seeds):
        atoms = Atoms(numbers=[79] * len(starts[c]), positions=starts[c])
        atoms.set_calculator(calc())
        ens = NUTSCanonicalEnsemble(atoms, temperature=300, seed=seed,
                                    escape_level=6)
        ch = bn.chains[c]
        # the initial step-size searches agree
        assert np.log(10 * ens.step_size) == pytest.approx(ch.mu, rel=1e-12)
        traj, meta = ens.run(iters)
        assert meta['accepted_samples'] == ch.metadata['accepted_samples']
        assert meta['samples_total'] == ch.metadata['samples_total']
        assert len(traj) - 1 == len(ch.samples)
        for a, x in zip(traj[1:], ch.samples):
            assert np.allclose(a.get_positions(), x, rtol=0, atol=1e-9)
        assert ens.step_size == pytest.approx(ch.step_size, rel=1e-9)
    assert bn.evaluations > 0


def test_single_evaluation_mode_runs_and_samples():
    from pyiid_gb300.nuts import BatchedNUTS
    from pyiid_gb300.sampling import PDFPotential
    s, target, starts, tab, calc = setup(chains=4)
    pot = PDFPotential([79] * len(starts[0]), target, dict(EXP), conv=50.,
                       n_configs=len(starts), table=tab)
    bn = BatchedNUTS(pot, np.stack(starts), temperature=300,
                     seeds=[1, 2, 3, 4], escape_level=6, exact=False)
    bn.step(3)
    assert sum(ch.metadata['accepted_samples'] for ch in bn.chains) > 0
    assert np.all(np.isfinite(bn.energies()))
