"""GPU parity at the benchmarked sizes, against the FP64 oracle.

The smaller parity tests pin every code path; these pin the same paths at
the sizes the samplers and the batched benchmark run:

* the adjoint potential gradient on a 1,000-atom fcc Au particle on the
  default experiment grid (Q_pdf step 0.0756865, 330 bins; r 0-40 step 0.01,
  4,000 points), for one configuration and for the 64-chain batch the
  batched HMC evaluates: Rw to 1e-5, complete gradient rows of 16 seeded
  atoms to 1e-4, central differences (h = 1e-4 A) of the FP64 oracle on 64
  seeded coordinates to 1e-4, and the reference's -1/2 convention through
  the compat chain get_grad_fq -> get_grad_pdf -> get_grad_rw at full size
  (calc/calc_1d.py:89-95, kernels/master_kernel.py:293-347);
* F(Q) of the 256 seeded Au/Pt alloys of 55-2,000 atoms in one batched
  launch (and its CUDA-graph replay): sampled bins of every configuration
  to 1e-5 (flat_multi_cpu_wrap.py:22-60 per configuration);
* single-atom Metropolis on one 1,000-atom chain on the default grid, every
  proposal against a full FP64 evaluation of the proposed configuration
  (sim/hmc.py:66-92's acceptance rule).

Tolerances are norm-wise relative, as in the other GPU tests.
"""
import numpy as np
import pytest

from oracle import debye_c as C
from oracle import debye_np as O
from oracle import mh_np
from pyiid_gb300 import structures as S

pytestmark = pytest.mark.gpu

TOL_F = 1e-5
TOL_G = 1e-4
N_AU = 1000


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


@pytest.fixture(scope='module')
def au1000():
    """The 1,000-atom Au particle of the HMC benchmark: reference
    (undisplaced) G(r) as gobs, displaced configurations seeds 4, 5, ..."""
    from pyiid_gb300.sampling import PDFPotential, experiment_grids
    exp, qb, nb, rg = experiment_grids(None)
    assert (nb, len(rg)) == (330, 4000)
    ref = S.fcc_nearest(4.08, N_AU).astype(np.float32)
    probe = PDFPotential([79] * N_AU, np.zeros(len(rg)), None)
    sp, tab = probe.species, probe.table
    f_ref = C.fq_all_bins(ref, sp, tab, qb)
    T = O.tmatrix(nb, exp['rstep'], qb, rg, exp['qmin'])
    gobs = f_ref @ T
    return {'exp': exp, 'qb': qb, 'nb': nb, 'rg': rg, 'ref': ref, 'sp': sp,
            'tab': tab, 'gobs': gobs, 'T': T}


def test_adjoint_gradient_at_1000_atoms_default_grid(au1000):
    import torch
    from pyiid_gb300.sampling import PDFPotential
    d = au1000
    x = S.displaced(d['ref'], 0.05, 4)
    pot = PDFPotential([79] * N_AU, d['gobs'], None, conv=1.0, n_configs=1)
    e, g = pot.evaluate(torch.as_tensor(x, device='cuda'))
    e = float(e[0].item())
    g = g.cpu().numpy().astype(np.float64)
    rng = np.random.default_rng(2024)
    atoms = np.sort(rng.choice(N_AU, 16, replace=False)).astype(np.int32)
    rows, (val, scale, gcalc, f, T) = C.true_grad_rows(
        x, d['sp'], d['tab'], d['exp'], d['qb'], d['gobs'], atoms,
        with_chain=True)
    assert 0.0 < val < 1.0 and scale > 0
    assert abs(e - val) <= TOL_F * abs(val), (e, val)
    assert rel(g[atoms], rows) <= TOL_G, rel(g[atoms], rows)

    # central differences of the FP64 oracle, h = 1e-4 A, 64 coordinates
    h = 1e-4
    s0 = C.pair_sums(x, d['sp'], d['tab'], d['qb'], np.arange(d['nb']))
    na = O.normalization(d['tab'][d['sp']])
    coords = rng.choice(3 * N_AU, 64, replace=False)
    fd = np.empty(64)
    for i, idx in enumerate(coords):
        a, c = divmod(int(idx), 3)
        rw = []
        for sgn in (1.0, -1.0):
            new = x[a].astype(np.float64)
            new[c] += sgn * h
            ds = C.moved_atom_sums(x, d['sp'], d['tab'], d['qb'], a, new)
            fp = 2 * np.nan_to_num((s0 + ds) / na)
            rw.append(O.get_rw(d['gobs'], fp @ T)[0])
        fd[i] = (rw[0] - rw[1]) / (2 * h)
    got = g.reshape(-1)[coords]
    assert rel(got, fd) <= TOL_G, rel(got, fd)


def test_compat_chain_is_minus_half_of_the_adjoint_at_1000_atoms(au1000):
    """get_grad_fq [1000, 3, 330] (rows of 16 atoms against the oracle),
    then get_grad_pdf [1000, 3, 4000] and get_grad_rw: the reference's
    convention, -1/2 of the true gradient the adjoint kernel returns."""
    import torch
    from pyiid_gb300 import debye as D
    from pyiid_gb300.sampling import PDFPotential
    d = au1000
    x = S.displaced(d['ref'], 0.05, 4)
    xt = torch.as_tensor(x, device='cuda')
    pot = PDFPotential([79] * N_AU, d['gobs'], None, conv=1.0, n_configs=1)
    _, g = pot.evaluate(xt)
    g = g.cpu().numpy().astype(np.float64)
    gcalc = pot.buffers()['gcalc'][0].clone()
    gq = D.grad_fq(xt, d['sp'], d['tab'], d['qb'])
    atoms = np.arange(0, N_AU, 67, dtype=np.int32)[:16]
    ds = C.grad_rows(x, d['sp'], d['tab'], d['qb'], atoms)
    na = O.normalization(d['tab'][d['sp']])
    want = np.nan_to_num(-ds / na)
    assert rel(gq.cpu().numpy()[atoms], want) <= TOL_G
    gp = D.grad_pdf(gq, d['qb'], d['exp']['rstep'], d['rg'],
                    d['exp']['qmin'])
    assert tuple(gp.shape) == (N_AU, 3, 4000)
    pg = D.potential_grad(gp, gcalc, torch.as_tensor(d['gobs'],
                                                     device='cuda'), 'rw')
    pg = pg.cpu().numpy()
    assert rel(-2.0 * pg, g) <= TOL_G, rel(-2.0 * pg, g)


def test_64_chain_batch_at_1000_atoms(au1000):
    """The batched evaluation the HMC benchmark replays: Rw of all 64
    configurations to 1e-5 and the gradient rows of two atoms per chain
    (128 rows) to 1e-4 against the FP64 oracle."""
    import torch
    from pyiid_gb300.sampling import PDFPotential
    d = au1000
    xs = np.stack([S.displaced(d['ref'], 0.05, 4 + c) for c in range(64)])
    pot = PDFPotential([79] * N_AU, d['gobs'], None, conv=1.0, n_configs=64)
    e, g = pot.evaluate(torch.as_tensor(xs.reshape(-1, 3), device='cuda'))
    e = e.cpu().numpy()
    g = g.cpu().numpy().astype(np.float64).reshape(64, N_AU, 3)
    rng = np.random.default_rng(64)
    got, want = [], []
    for c in range(64):
        atoms = np.sort(rng.choice(N_AU, 2, replace=False)).astype(np.int32)
        rows, chain = C.true_grad_rows(xs[c], d['sp'][:N_AU], d['tab'],
                                       d['exp'], d['qb'], d['gobs'], atoms,
                                       with_chain=True)
        val = chain[0]
        assert abs(e[c] - val) <= TOL_F * abs(val), (c, e[c], val)
        got.append(g[c, atoms])
        want.append(rows)
    assert rel(np.concatenate(got), np.concatenate(want)) <= TOL_G


def test_256_alloys_batched_fq_sampled_bins():
    """Configuration set of the batched benchmark (256 fcc Au/Pt random
    alloys, N ~ U{55..2000}, a = 4.0, sigma 0.05, Q 0.1-25 step 0.05): one
    pyiid_batch_fq launch, and its CUDA-graph replay bit for bit; 8 sampled
    bins (the first and last returned ones included) of every configuration
    against FP64 pair sums."""
    import torch
    import bench
    from pyiid_gb300 import debye as D
    pos, sp, off, tab, sizes = bench.batched_workload()
    assert len(sizes) == 256 and sizes.min() >= 55 and sizes.max() <= 2000
    p = torch.as_tensor(pos, device='cuda')
    out = torch.empty((256, 500), dtype=torch.float32, device='cuda')
    D.batch_fq(p, sp, off, tab, 0.05, 2, out=out)
    eager = out.clone()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        D.batch_fq(p, sp, off, tab, 0.05, 2, out=out)
    torch.cuda.current_stream().wait_stream(s)
    graph = torch.cuda.CUDAGraph()
    out.zero_()
    with torch.cuda.graph(graph):
        D.batch_fq(p, sp, off, tab, 0.05, 2, out=out)
    out.zero_()
    graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(out, eager)
    f = eager.cpu().numpy()
    assert np.all(f[:, :2] == 0)
    rng = np.random.default_rng(256)
    worst = 0.0
    for b in range(256):
        o0, o1 = int(off[b]), int(off[b + 1])
        bins = np.unique(np.concatenate(
            [[2, 499], rng.choice(np.arange(3, 499), 6, replace=False)]
        )).astype(np.int32)
        ssum = C.pair_sums(pos[o0:o1], sp[o0:o1], tab, 0.05, bins)
        na = O.normalization(tab[sp[o0:o1]])[bins]
        want = 2 * np.nan_to_num(ssum / na)
        err = rel(f[b, bins], want)
        worst = max(worst, err)
        assert err <= TOL_F, (b, int(sizes[b]), err)
    print(f'256 alloys: worst sampled-bin error {worst:.2e}')


def test_single_atom_mh_at_1000_atoms_every_proposal(au1000):
    """One 1,000-atom Au chain (E = 100 Rw, 300 K, sigma 0.1 A, the
    delayed-acceptance benchmark's moves) on the default grid: every
    proposal is the oracle generator's, its proposed Rw equals a full FP64
    evaluation of the proposed configuration (1e-5), its energy change
    agrees with the oracle's, every decision is the Metropolis rule's, and
    the final positions are the replayed ones."""
    import torch
    from pyiid_gb300.sampling import PDFPotential, SingleAtomMC
    d = au1000
    conv, temp, sigma, seed = 100.0, 300.0, 0.1, 31
    x0 = S.displaced(d['ref'], 0.05, 4).astype(np.float32)
    pot = PDFPotential([79] * N_AU, d['gobs'], None, conv=conv, n_configs=1)
    mc = SingleAtomMC(pot, x0, temperature=temp, sigma=sigma, seed=seed,
                      resync_every=None)
    n_steps = 24
    trace = torch.empty((n_steps, 1, 8), dtype=torch.float64, device='cuda')
    mc.step(n_steps, trace=trace)
    tr = trace.cpu().numpy()[:, 0]
    x = x0.copy()
    v = C.potential_chain(x, d['sp'], d['tab'], d['exp'], d['qb'],
                          d['gobs'])[0]
    n_acc = 0
    dv_err = 0.0
    for t in range(n_steps):
        rec = tr[t]
        atom, dxyz, logu = mh_np.proposal(seed, 0, t, N_AU, sigma)
        assert int(rec[0]) == atom
        assert np.allclose(rec[1:4] - x[atom], dxyz, atol=2e-6)
        assert abs(rec[4] - logu) <= 2e-7 * abs(logu) + 1e-7
        xp = x.copy()
        xp[atom] = rec[1:4].astype(np.float32)
        vp = C.potential_chain(xp, d['sp'], d['tab'], d['exp'], d['qb'],
                               d['gobs'])[0]
        assert abs(rec[5] - vp) <= TOL_F * abs(vp), (t, rec[5], vp)
        assert abs(rec[7] - v) <= TOL_F * abs(v), (t, rec[7], v)
        dv_err = max(dv_err, abs((rec[5] - rec[7]) - (vp - v)))
        z = logu + conv * (vp - v) / mc.kT
        if abs(z) > 1e-2:
            assert bool(rec[6]) == (z < 0), (t, z)
        if rec[6]:
            x, v = xp, vp
            n_acc += 1
    assert 0 < n_acc < n_steps
    # the energy changes the decisions rest on, in units of kT
    print(f'1,000-atom MH: {n_acc}/{n_steps} accepted, max energy-change '
          f'error {conv * dv_err / mc.kT:.2e} kT')
    assert conv * dv_err / mc.kT <= 1e-3, conv * dv_err / mc.kT
    assert np.array_equal(mc.positions().cpu().numpy(), x)
    e = float(mc.state['energy'][0, 0].item())
    assert abs(e - v) <= TOL_F * abs(v)
