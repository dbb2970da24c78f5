"""Host-chosen moves with O(N K) exact energies (pyiid_mc_propose /
pyiid_mc_accept) and the grand-canonical ensemble built on them."""
import numpy as np
import pytest

from oracle import debye_np as O
from oracle import mh_np
from pyiid_gb300 import structures as S
from pyiid_gb300.scatter_factors import form_factor_array

pytestmark = pytest.mark.gpu

EXP = {'qmin': 0.6, 'qmax': 22.0, 'rmin': 0.5, 'rmax': 14.0, 'rstep': 0.02}


def setup(sizes, seed=0):
    from pyiid_gb300.sampling import PDFPotential, experiment_grids
    exp, qb, nb, rg = experiment_grids(EXP)
    ref = S.displaced(S.fcc_nearest(4.08, 40), 0.0, 0)
    tab = form_factor_array(79, np.arange(nb) * qb)[None].astype(np.float32)
    gobs = O.pdf_tmatrix(O.fq(ref, np.repeat(tab, 40, 0), qb), exp['rstep'],
                         qb, rg, exp['qmin'])
    rng = np.random.default_rng(seed)
    numbers = [rng.choice([78, 79], size=n) for n in sizes]
    xs = [S.displaced(S.fcc_nearest(4.08, n), 0.05, seed + c)
          for c, n in enumerate(sizes)]
    pot = PDFPotential(numbers, gobs, EXP, conv=1.0)
    return pot, [x.astype(np.float32) for x in xs], exp, gobs


def packed(pot, xs, species):
    off = np.concatenate([[0], np.cumsum([len(x) for x in xs])])
    return np.concatenate(xs).astype(np.float32), np.concatenate(species), off


def test_every_move_type_matches_oracle_and_commits_consistently():
    import torch
    from pyiid_gb300 import debye
    pot, xs, exp, gobs = setup([30, 25, 33], seed=2)
    species = [pot.species[pot.offsets[c]:pot.offsets[c + 1]].copy()
               for c in range(3)]
    rng = np.random.default_rng(7)
    for rnd in range(3):
        x, sp, off = packed(pot, xs, species)
        xt = torch.as_tensor(x, device='cuda')
        st = debye.mh_init(xt, sp, off, pot.table, pot.qstep,
                           pot.exp['rstep'], pot.rgrid, pot.exp['qmin'],
                           pot.gobs)
        # chain 0 inserts, chain 1 removes, chain 2 displaces
        mode = [debye.MOVE_INSERT, debye.MOVE_REMOVE, debye.MOVE_DISPLACE]
        atom = [0, int(rng.integers(len(xs[1]))), int(rng.integers(len(xs[2])))]
        xyz = np.stack([rng.uniform(-6, 6, 3),
                        np.zeros(3),
                        xs[2][atom[2]] + rng.normal(0, 0.2, 3)]).astype(np.float32)
        new_sp = [int(rng.integers(2)), 0, 0]
        ev = debye.mc_propose(xt, sp, off, pot.table, pot.qstep,
                              pot.exp['rstep'], pot.rgrid, pot.exp['qmin'],
                              st, mode, atom, xyz, new_sp).cpu().numpy()
        proposed = []
        for c in range(3):
            x1, s1 = xs[c].copy(), species[c].copy()
            if mode[c] == debye.MOVE_INSERT:
                x1 = np.vstack([x1, xyz[c]])
                s1 = np.append(s1, new_sp[c])
            elif mode[c] == debye.MOVE_REMOVE:
                x1 = np.delete(x1, atom[c], axis=0)
                s1 = np.delete(s1, atom[c])
            else:
                x1[atom[c]] = xyz[c]
            v = mh_np.potential_of(x1, s1, pot.table, exp, gobs)
            assert abs(ev[c, 0] - v) <= 1e-5 * v, (rnd, c, ev[c, 0], v)
            proposed.append((x1.astype(np.float32), s1))
        # accept chains 0 and 2, reject 1; the state must equal a fresh
        # evaluation of the resulting configurations
        acc = [True, False, True]
        debye.mc_accept(st, acc)
        for c in range(3):
            if acc[c]:
                xs[c], species[c] = proposed[c]
        x2, sp2, off2 = packed(pot, xs, species)
        fresh = debye.mh_init(torch.as_tensor(x2, device='cuda'), sp2, off2,
                              pot.table, pot.qstep, pot.exp['rstep'],
                              pot.rgrid, pot.exp['qmin'], pot.gobs)
        vr, vf = debye.mh_views(st), debye.mh_views(fresh)
        for key, tol in (('S', 1e-6), ('F', 1e-6)):
            a, b = vr[key].cpu().numpy(), vf[key].cpu().numpy()
            assert np.abs(a - b).max() <= tol * np.abs(b).max(), (rnd, key)
        e_run = st['energy'][:, 0].cpu().numpy()
        e_new = fresh['energy'][:, 0].cpu().numpy()
        assert np.all(np.abs(e_run - e_new) <= 1e-5 * e_new), (rnd, e_run, e_new)


def test_invalid_moves_are_rejected_with_messages():
    import torch
    from pyiid_gb300 import debye
    from pyiid_gb300._native import NativeError
    pot, xs, exp, gobs = setup([10, 1], seed=3)
    x, sp, off = packed(pot, xs, [pot.species[:10], pot.species[10:]])
    xt = torch.as_tensor(x, device='cuda')
    st = debye.mh_init(xt, sp, off, pot.table, pot.qstep, pot.exp['rstep'],
                       pot.rgrid, pot.exp['qmin'], pot.gobs)
    args = (xt, sp, off, pot.table, pot.qstep, pot.exp['rstep'], pot.rgrid,
            pot.exp['qmin'], st)
    z = np.zeros((2, 3), np.float32)
    with pytest.raises(NativeError, match='removal'):
        debye.mc_propose(*args, [debye.MOVE_DISPLACE, debye.MOVE_REMOVE],
                         [0, 0], z, [0, 0])
    with pytest.raises(NativeError, match='atom'):
        debye.mc_propose(*args, [debye.MOVE_DISPLACE, debye.MOVE_DISPLACE],
                         [10, 0], z, [0, 0])
    with pytest.raises(NativeError, match='new_species'):
        debye.mc_propose(*args, [debye.MOVE_INSERT, debye.MOVE_DISPLACE],
                         [0, 0], z, [5, 0])
    with pytest.raises(NativeError, match='mode'):
        debye.mc_propose(*args, [7, debye.MOVE_DISPLACE], [0, 0], z, [0, 0])


def _gcmc_run(incremental, seed, steps):
    from pyiid_gb300.atoms import Atoms
    from pyiid_gb300.calc.calc_1d import Calc1D
    from pyiid_gb300.experiments.elasticscatter import ElasticScatter
    from pyiid_gb300.sim.gcmc import GrandCanonicalEnsemble
    s = ElasticScatter(exp_dict={'qmin': 0.6, 'qmax': 20.0, 'rmax': 12.0,
                                 'rstep': 0.02})
    ref = Atoms(numbers=[79] * 38, positions=S.fcc_nearest(4.08, 38))
    target = s.get_pdf(ref)
    atoms = Atoms(numbers=[79] * 30,
                  positions=S.displaced(S.fcc_nearest(4.08, 30), 0.05, 1))
    atoms.set_cell(np.eye(3) * 6.0)
    atoms.set_calculator(Calc1D(target_data=target, exp_function=s.get_pdf,
                                exp_grad_function=s.get_grad_pdf, conv=30.))
    np.random.seed(seed)
    gc = GrandCanonicalEnsemble(atoms, {'Au': 0.1}, temperature=2000,
                                seed=seed, incremental=incremental)
    assert (gc._engine is not None) == bool(incremental)
    traj, meta = gc.run(steps)
    return traj, meta


def test_gcmc_incremental_engine_reproduces_the_reference_algorithm():
    """Same seeds: the O(N K) engine makes the same proposals and the same
    decisions as the reference algorithm (full energy of every trial
    configuration through Calc1D), so the trajectories coincide."""
    t_ref, m_ref = _gcmc_run(False, 5, 30)
    t_inc, m_inc = _gcmc_run(True, 5, 30)
    for k in ('accepted_additions', 'rejected_additions',
              'accepted_removals', 'rejected_removals'):
        assert m_ref[k] == m_inc[k], (k, m_ref, m_inc)
    assert m_ref['accepted_additions'] + m_ref['accepted_removals'] > 0
    assert len(t_ref) == len(t_inc)
    for a, b in zip(t_ref, t_inc):
        assert len(a) == len(b)
        assert np.allclose(a.get_positions(), b.get_positions(), atol=1e-6)
    # the engine's energy of the final state equals a full evaluation
    last = t_inc[-1]
    e_engine = last.get_potential_energy()
    last.get_calculator().results = {}
    last.get_calculator().atoms = None
    e_full = last.get_potential_energy()
    assert abs(e_engine - e_full) <= 1e-5 * abs(e_full)
