"""Device-resident potential, autograd adjoint, batched HMC and the
pyiid.sim samplers on the GPU."""
import numpy as np
import pytest

from oracle import debye_np as O
from pyiid_gb300 import structures as S
from pyiid_gb300.scatter_factors import form_factor_array

pytestmark = pytest.mark.gpu

EXP = {'qmin': 0.6, 'qmax': 22.0, 'rmin': 0.5, 'rmax': 14.0, 'rstep': 0.02}


def setup(nconf=3, n=40, seed=0):
    import torch
    from pyiid_gb300.sampling import PDFPotential, experiment_grids
    exp, qb, nb, rg = experiment_grids(EXP)
    ref = S.displaced(S.fcc_nearest(4.08, n), 0.0, 0)
    tab = form_factor_array(79, np.arange(nb) * qb)[None].astype(np.float32)
    gobs = O.pdf_tmatrix(O.fq(ref, np.repeat(tab, n, 0), qb), exp['rstep'],
                         qb, rg, exp['qmin'])
    pot = PDFPotential([79] * n, gobs, EXP, conv=100.0, n_configs=nconf)
    xs = np.stack([S.displaced(S.fcc_nearest(4.08, n), 0.05, seed + c)
                   for c in range(nconf)])
    return pot, xs, exp, tab, gobs, torch


def test_potential_and_autograd_match_oracle():
    pot, xs, exp, tab, gobs, torch = setup()
    from pyiid_gb300.sampling import potential_energy
    x = torch.as_tensor(xs.reshape(-1, 3), device='cuda').requires_grad_(True)
    e = potential_energy(x, pot)
    (e * torch.arange(1, 4, device='cuda', dtype=e.dtype)).sum().backward()
    g = x.grad.cpu().numpy().reshape(xs.shape)
    n = xs.shape[1]
    for c in range(3):
        val, tg = O.true_grad_potential(xs[c], np.repeat(tab, n, 0), exp, gobs)
        assert abs(e[c].item() - 100 * val) <= 1e-5 * 100 * val
        err = np.linalg.norm(g[c] - 100 * (c + 1) * tg) / np.linalg.norm(
            100 * (c + 1) * tg)
        assert err < 1e-4, err


def test_adjoint_gradient_vs_central_differences():
    """Central FD (h = 1e-4 A) of the FP64 oracle energy, 24 coordinates."""
    pot, xs, exp, tab, gobs, torch = setup(nconf=1, n=30)
    x = torch.as_tensor(xs.reshape(-1, 3), device='cuda')
    _, g = pot.evaluate(x)
    g = g.cpu().numpy() / 100.0
    x64 = xs[0].astype(np.float64)
    per_atom = np.repeat(tab, 30, 0)
    rng = np.random.default_rng(3)
    idx = [(int(a), int(c)) for a, c in zip(rng.integers(0, 30, 24),
                                           rng.integers(0, 3, 24))]
    h = 1e-4
    fd, an = [], []
    for a, c in idx:
        xp, xm = x64.copy(), x64.copy()
        xp[a, c] += h
        xm[a, c] -= h
        fd.append((O.potential_value(xp, per_atom, exp, gobs, cast32=False) -
                   O.potential_value(xm, per_atom, exp, gobs, cast32=False))
                  / (2 * h))
        an.append(g[a, c])
    fd, an = np.array(fd), np.array(an)
    assert np.linalg.norm(fd - an) / np.linalg.norm(fd) < 1e-4


def test_hmc_graph_equals_eager_and_moves():
    from pyiid_gb300.sampling import BatchedHMC
    pot, xs, exp, tab, gobs, torch = setup(nconf=4, n=40)
    a = BatchedHMC(pot, xs, temperature=300, dt=2e-2, n_steps=5, seed=7,
                   graph=False)
    a.step(6)
    xa = a.positions().cpu().numpy()
    b = BatchedHMC(pot, xs, temperature=300, dt=2e-2, n_steps=5, seed=7,
                   graph=True)
    b.x.copy_(torch.as_tensor(xs.reshape(-1, 3), device='cuda'))
    b.u.copy_(a.pot.evaluate(torch.as_tensor(xs.reshape(-1, 3),
                                             device='cuda'))[0])
    b.g.copy_(a.pot.evaluate(torch.as_tensor(xs.reshape(-1, 3),
                                             device='cuda'))[1])
    b.gen.manual_seed(7)
    b.accepted.zero_()
    b.step(6)
    xb = b.positions().cpu().numpy()
    assert np.array_equal(xa, xb)
    assert np.array_equal(a.acceptance(), b.acceptance())
    assert not np.allclose(xa, xs.reshape(-1, 3))
    acc = a.acceptance()
    assert np.all((acc >= 0) & (acc <= 1)) and acc.mean() > 0


def test_leapfrog_reversible_on_device():
    pot, xs, exp, tab, gobs, torch = setup(nconf=2, n=40)
    m = torch.as_tensor(pot.masses, dtype=torch.float64, device='cuda')[:, None]
    x0 = torch.as_tensor(xs.reshape(-1, 3), device='cuda')
    p0 = torch.randn(x0.shape, dtype=torch.float64, device='cuda', generator=
                     torch.Generator(device='cuda').manual_seed(1)) * 0.02
    dt = 1e-2

    def run(x, p, n):
        x = x.clone()
        p = p.clone()
        _, g = pot.evaluate(x)
        for _ in range(n):
            p = p - 0.5 * dt * g.double()
            x = (x.double() + dt * p / m).float()
            _, g = pot.evaluate(x)
            p = p - 0.5 * dt * g.double()
        return x, p

    x1, p1 = run(x0, p0, 8)
    x2, p2 = run(x1, -p1, 8)
    assert torch.max(torch.abs(x2 - x0)).item() < 2e-5


def test_reference_sim_api_with_gb300_calculator():
    """pyiid/tests/test_sim: leapfrog reversibility (test_leapfrog.py:58-73),
    NUTS lowers the potential (test_nuts.py:64), dynamics and HMC run."""
    from pyiid_gb300.atoms import Atoms, MaxwellBoltzmannDistribution, kB
    from pyiid_gb300.calc.calc_1d import Calc1D
    from pyiid_gb300.experiments.elasticscatter import ElasticScatter
    from pyiid_gb300.sim import leapfrog
    from pyiid_gb300.sim.dynamics import classical_dynamics
    from pyiid_gb300.sim.nuts_hmc import NUTSCanonicalEnsemble
    from pyiid_gb300.sim.hmc import run_hmc
    s = ElasticScatter(dict(EXP))
    ideal = Atoms('Au20', S.fcc_nearest(4.08, 20))
    target = s.get_pdf(ideal)
    atoms = Atoms('Au20', S.displaced(S.fcc_nearest(4.08, 20), 0.1, 5))
    atoms.set_calculator(Calc1D(target_data=target, exp_function=s.get_pdf,
                                exp_grad_function=s.get_grad_pdf, conv=30))
    MaxwellBoltzmannDistribution(atoms, 300 * kB, force_temp=True,
                                 rng=np.random.default_rng(2))
    a1 = leapfrog(atoms, 0.5, center=False)
    a1.set_momenta(-a1.get_momenta())
    a2 = leapfrog(a1, 0.5, center=False)
    assert np.allclose(a2.positions, atoms.positions, atol=1e-5)
    traj = classical_dynamics(atoms, 0.5, 3)
    assert len(traj) == 4
    start = atoms.get_potential_energy()
    nuts = NUTSCanonicalEnsemble(atoms, temperature=300, escape_level=4,
                                 seed=3)
    traj, meta = nuts.run(4)
    pes = [a.get_potential_energy() for a in traj]
    assert min(pes) <= start
    assert meta['seed'] == 3
    tr, acc, num = run_hmc(atoms, 3, 0.5, 3, .9, .5, .65, 1.05, .95, .01, 5.,
                           rng=np.random.RandomState(4))
    assert len(acc) == 3
