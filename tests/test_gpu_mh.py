"""Single-atom Metropolis chains with O(N K) exact energy changes
(pyiid_mh_init / pyiid_mh_steps) against the FP64 oracle, proposal by
proposal."""
import numpy as np
import pytest

from oracle import debye_np as O
from oracle import mh_np
from pyiid_gb300 import structures as S
from pyiid_gb300.scatter_factors import form_factor_array

pytestmark = pytest.mark.gpu

EXP = {'qmin': 0.6, 'qmax': 22.0, 'rmin': 0.5, 'rmax': 14.0, 'rstep': 0.02}
CONV = 100.0


def make_potential(sizes, alloy, seed=0, exp_dict=EXP):
    from pyiid_gb300.sampling import PDFPotential, experiment_grids
    exp, qb, nb, rg = experiment_grids(exp_dict)
    ref = S.displaced(S.fcc_nearest(4.08, 40), 0.0, 0)
    tab = form_factor_array(79, np.arange(nb) * qb)[None].astype(np.float32)
    gobs = O.pdf_tmatrix(O.fq(ref, np.repeat(tab, 40, 0), qb), exp['rstep'],
                         qb, rg, exp['qmin'])
    rng = np.random.default_rng(seed)
    numbers, xs = [], []
    for c, n in enumerate(sizes):
        if alloy:
            numbers.append(rng.choice([78, 79], size=n))
        else:
            numbers.append(np.full(n, 79))
        xs.append(S.displaced(S.fcc_nearest(4.08, n), 0.05, seed + c)
                  if n else np.zeros((0, 3)))
    pot = PDFPotential(numbers, gobs, exp_dict, conv=CONV)
    return pot, np.concatenate(xs).astype(np.float32), exp, gobs


def oracle_potential(pot, exp, gobs, x, c):
    o0, o1 = pot.offsets[c], pot.offsets[c + 1]
    return mh_np.potential_of(x[o0:o1], pot.species[o0:o1], pot.table, exp,
                              gobs)


def test_trace_matches_oracle_step_by_step():
    """Every proposal (atom, displacement, log u) is the oracle generator's,
    every proposed potential is the oracle's full re-evaluation of the
    proposed configuration (1e-5), every decision is the Metropolis rule's,
    and the final state equals the oracle's."""
    import torch
    from pyiid_gb300.sampling import SingleAtomMC
    sizes = [40, 30, 1, 0, 25]
    pot, x0, exp, gobs = make_potential(sizes, alloy=True)
    seed, sigma, temp = 11, 0.15, 3000.0
    mc = SingleAtomMC(pot, x0, temperature=temp, sigma=sigma, seed=seed,
                      resync_every=None)
    n_steps = 8
    trace = torch.empty((n_steps, len(sizes), 8), dtype=torch.float64,
                        device='cuda')
    mc.step(n_steps, trace=trace)
    tr = trace.cpu().numpy()
    x = x0.astype(np.float32).copy()
    v = [oracle_potential(pot, exp, gobs, x, c) if sizes[c] > 1 else np.nan
         for c in range(len(sizes))]
    checked = 0
    for t in range(n_steps):
        for c, n in enumerate(sizes):
            rec = tr[t, c]
            if n < 2:
                assert np.all(rec == 0)
                continue
            atom, d, logu = mh_np.proposal(seed, c, t, n, sigma)
            assert int(rec[0]) == atom
            g = pot.offsets[c] + atom
            assert np.allclose(rec[1:4] - x[g], d, atol=2e-6)
            assert abs(rec[4] - logu) <= 2e-7 * abs(logu) + 1e-7
            xp = x.copy()
            xp[g] = rec[1:4].astype(np.float32)
            vp = oracle_potential(pot, exp, gobs, xp, c)
            assert abs(rec[5] - vp) <= 1e-5 * abs(vp), (t, c, rec[5], vp)
            assert abs(rec[7] - v[c]) <= 1e-5 * abs(v[c])
            z = logu + CONV * (vp - v[c]) / mc.kT
            if abs(z) > 1e-2:
                assert bool(rec[6]) == (z < 0), (t, c, z)
            if rec[6]:
                x = xp
                v[c] = vp
            checked += 1
    assert checked == n_steps * 3
    acc = tr[:, [0, 1, 4], 6]
    assert 0 < acc.sum() < acc.size  # the case exercises both outcomes
    # final state: positions exactly as replayed, energies and sums as the
    # oracle's full evaluation
    assert np.array_equal(mc.positions().cpu().numpy(), x)
    e = mc.state['energy'][:, 0].cpu().numpy()
    for c in (0, 1, 4):
        assert abs(e[c] - v[c]) <= 1e-5 * v[c]
    sr = mc.sums().cpu().numpy()
    kmin = int(np.ceil(EXP['qmin'] / pot.qstep))
    for c in (0, 1, 4):
        o0, o1 = pot.offsets[c], pot.offsets[c + 1]
        ref = mh_np.raw_sums(x[o0:o1], pot.species[o0:o1], pot.table,
                             pot.qstep)
        assert np.all(sr[c, :kmin] == 0)
        err = np.abs(sr[c, kmin:] - ref[kmin:]).max() / np.abs(ref).max()
        assert err < 1e-5, err
    cnt = mc.state['counter'].cpu().numpy()
    assert np.all(cnt == n_steps)


def test_zero_displacement_is_always_accepted_and_exact():
    """sigma = 0: the old and new pair terms are bitwise equal, so the
    proposed potential equals the current one exactly and every proposal is
    accepted without changing anything."""
    from pyiid_gb300.sampling import SingleAtomMC
    pot, x0, exp, gobs = make_potential([50, 33], alloy=True, seed=3)
    mc = SingleAtomMC(pot, x0, temperature=300, sigma=0.0, seed=1,
                      resync_every=None)
    from pyiid_gb300 import debye
    e0 = mc.state['energy'].clone()
    v0 = {k: debye.mh_views(mc.state)[k].clone() for k in ('S', 'F', 'uqe')}
    mc.step(21)
    assert np.all(mc.state['accepted'].cpu().numpy() == 21)
    assert np.array_equal(mc.positions().cpu().numpy(), x0)
    assert bool((mc.state['energy'] == e0).all())
    v1 = debye.mh_views(mc.state)
    for k, t in v0.items():
        assert bool((v1[k] == t).all()), k
    # an odd number of acceptances leaves the chains on the second buffer
    assert bool((v1['cur'] == 1).all())


def test_graph_replay_equals_eager():
    from pyiid_gb300.sampling import SingleAtomMC
    pot, x0, exp, gobs = make_potential([64, 48, 80], alloy=True, seed=5)
    a = SingleAtomMC(pot, x0, temperature=600, sigma=0.1, seed=21,
                     resync_every=None)
    a.step(96)
    b = SingleAtomMC(pot, x0, temperature=600, sigma=0.1, seed=21,
                     graph=True, steps_per_replay=16, resync_every=None)
    b.step(96)
    assert np.array_equal(a.positions().cpu().numpy(),
                          b.positions().cpu().numpy())
    assert bool((a.state['energy'] == b.state['energy']).all())
    assert bool((a.state['accepted'] == b.state['accepted']).all())
    assert a.state['accepted'].sum().item() > 0


def test_running_sums_do_not_drift():
    """3000 steps without re-synchronisation: the running sums and energies
    equal a fresh full evaluation of the final positions."""
    from pyiid_gb300 import debye
    from pyiid_gb300.sampling import SingleAtomMC
    pot, x0, exp, gobs = make_potential([200] * 8, alloy=False, seed=7)
    mc = SingleAtomMC(pot, x0, temperature=300, sigma=0.03, seed=2,
                      graph=True, steps_per_replay=100, resync_every=None)
    mc.step(3000)
    acc = mc.state['accepted'].cpu().numpy()
    assert acc.min() > 30, acc
    fresh = debye.mh_init(mc.x, pot.species, pot.offsets, pot.table,
                          pot.qstep, pot.exp['rstep'], pot.rgrid,
                          pot.exp['qmin'], pot.gobs, state={})
    s_run = mc.sums().cpu().numpy()
    s_new = debye.mh_views(fresh)['S'].cpu().numpy()
    f_run = debye.mh_views(mc.state)['F'].cpu().numpy()
    f_new = debye.mh_views(fresh)['F'].cpu().numpy()
    assert np.abs(f_run - f_new).max() <= 1e-6 * np.abs(f_new).max()
    q_run = debye.mh_views(mc.state)['uqe'].cpu().numpy()
    q_new = debye.mh_views(fresh)['uqe'].cpu().numpy()
    # u and q to 1e-6; ee (a difference of totals, tracked by increments)
    # to 1e-5 of itself
    assert np.all(np.abs(q_run[:, :2] - q_new[:, :2]) <= 1e-6 * np.abs(q_new[:, :2]))
    assert np.all(np.abs(q_run[:, 2] - q_new[:, 2]) <= 1e-5 * np.abs(q_new[:, 2]))
    err = np.abs(s_run - s_new).max() / np.abs(s_new).max()
    assert err < 1e-6, err
    e_run = mc.state['energy'][:, 0].cpu().numpy()
    e_new = fresh['energy'][:, 0].cpu().numpy()
    assert np.all(np.abs(e_run - e_new) <= 1e-5 * e_new)


def test_cold_chain_only_moves_downhill():
    import torch
    from pyiid_gb300.sampling import SingleAtomMC
    pot, x0, exp, gobs = make_potential([60, 60], alloy=False, seed=9)
    mc = SingleAtomMC(pot, x0, temperature=1e-7, sigma=0.05, seed=4,
                      resync_every=None)
    tr = torch.empty((40, 2, 8), dtype=torch.float64, device='cuda')
    mc.step(40, trace=tr)
    t = tr.cpu().numpy()
    vp, acc, v = t[..., 5], t[..., 6].astype(bool), t[..., 7]
    assert np.array_equal(acc, vp < v)
    assert acc.any()
    assert np.all(np.diff(t[..., 7], axis=0) <= 0)


def test_default_grid_without_qmin():
    """qmin = 0 (the bins from Q = 0 enter the transform)."""
    import torch
    from pyiid_gb300.sampling import SingleAtomMC
    exp_dict = {'qmin': 0.0, 'qmax': 25.0, 'rmin': 0.0, 'rmax': 40.0,
                'rstep': 0.01}
    pot, x0, exp, gobs = make_potential([45], alloy=False, seed=2,
                                        exp_dict=exp_dict)
    mc = SingleAtomMC(pot, x0, temperature=3000, sigma=0.1, seed=8,
                      resync_every=None)
    tr = torch.empty((4, 1, 8), dtype=torch.float64, device='cuda')
    mc.step(4, trace=tr)
    t = tr.cpu().numpy()
    x = x0.copy()
    for s in range(4):
        g = int(t[s, 0, 0])
        xp = x.copy()
        xp[g] = t[s, 0, 1:4].astype(np.float32)
        vp = oracle_potential(pot, exp, gobs, xp, 0)
        assert abs(t[s, 0, 5] - vp) <= 1e-5 * vp
        if t[s, 0, 6]:
            x = xp


def test_invalid_arguments_raise():
    import torch
    from pyiid_gb300 import debye
    from pyiid_gb300._native import NativeError
    pot, x0, exp, gobs = make_potential([20], alloy=False)
    x = torch.as_tensor(x0, device='cuda')
    st = debye.mh_init(x, pot.species, pot.offsets, pot.table, pot.qstep,
                       pot.exp['rstep'], pot.rgrid, pot.exp['qmin'], pot.gobs)
    args = (x, pot.species, pot.offsets, pot.table, pot.qstep,
            pot.exp['rstep'], pot.rgrid, pot.exp['qmin'], st, 1)
    with pytest.raises(NativeError, match='kT'):
        debye.mh_steps(*args, conv=1.0, kT=0.0, sigma=0.1, seed=0)
    with pytest.raises(NativeError, match='sigma'):
        debye.mh_steps(*args, conv=1.0, kT=1.0, sigma=-1.0, seed=0)
    with pytest.raises(NativeError, match='n_steps'):
        debye.mh_steps(x, pot.species, pot.offsets, pot.table, pot.qstep,
                       pot.exp['rstep'], pot.rgrid, pot.exp['qmin'], st, -1,
                       conv=1.0, kT=1.0, sigma=0.1, seed=0)


def test_gram_form_equals_transform_path():
    """The potential of mh_init (Gram form, no G(r)) equals the fused
    F -> G -> potential path of pyiid_batch_potential_grad."""
    import torch
    from pyiid_gb300 import debye
    for kind in ('rw', 'chi_sq'):
        pot, x0, exp, gobs = make_potential([40, 33, 57], alloy=True, seed=4)
        pot.kind = kind
        x = torch.as_tensor(x0, device='cuda')
        st = debye.mh_init(x, pot.species, pot.offsets, pot.table, pot.qstep,
                           pot.exp['rstep'], pot.rgrid, pot.exp['qmin'],
                           pot.gobs, kind=kind)
        e_ref, _ = pot.evaluate(x, want_grad=False)
        e_ref = e_ref.cpu().numpy() / pot.conv
        e = st['energy'][:, 0].cpu().numpy()
        assert np.allclose(e, e_ref, rtol=1e-6, atol=0), (kind, e, e_ref)
        sc = st['energy'][:, 1].cpu().numpy()
        sc_ref = pot.buffers()['energy'][:, 1].cpu().numpy()
        assert np.allclose(sc, sc_ref, rtol=1e-6, atol=0)
