"""The drop-in samplers (pyiid_gb300.sim) on the CPU with a plain-Python
harmonic calculator: the reference's leapfrog checks
(pyiid/tests/test_sim/test_leapfrog.py: no momentum, momentum,
reversibility), dynamics lowering the energy both ways in time
(test_sim/test_dynamics.py), energy conservation, and seeded
reproducibility of HMC and NUTS
(test_sim/test_nuts.py runs NUTS on the scattering calculator; that run is
in tests/test_gpu_sampling.py)."""
import numpy as np

from pyiid_gb300.atoms import Atoms, Calculator
from pyiid_gb300.sim import leapfrog
from pyiid_gb300.sim.dynamics import classical_dynamics
from pyiid_gb300.sim.hmc import run_hmc
from pyiid_gb300.sim.nuts_hmc import NUTSCanonicalEnsemble


class _Well(Calculator):
    """E = k/2 sum |x - x0|^2, forces -k (x - x0)."""
    implemented_properties = ['energy', 'forces']

    def __init__(self, k=1.0, x0=None, **kw):
        Calculator.__init__(self, **kw)
        self.k = float(k)
        self.x0 = None if x0 is None else np.array(x0, float)

    def calculate(self, atoms=None, properties=['energy'],
                  system_changes=()):
        Calculator.calculate(self, atoms, properties, system_changes)
        x = self.atoms.positions
        d = x - (self.x0 if self.x0 is not None else 0.0)
        self.results['energy'] = 0.5 * self.k * float((d * d).sum())
        self.results['forces'] = -self.k * d


def _square(k=1.0, x0=None):
    a = Atoms('Au4', [[0, 0, 0], [3, 0, 0], [0, 3, 0], [3, 3, 0]])
    a.set_calculator(_Well(k, x0))
    return a


def test_leapfrog_without_force_or_momentum_stays_put():
    a = _square(k=0.0)
    b = leapfrog(a, 1, False)
    assert np.array_equal(a.positions, b.positions)


def test_leapfrog_with_momentum_drifts_by_the_velocity():
    a = _square(k=0.0)
    a.set_momenta(np.ones((len(a), 3)))
    b = leapfrog(a, 1, False)
    assert np.allclose(b.positions - a.get_velocities(), a.positions,
                       rtol=0, atol=1e-12)


def test_leapfrog_is_reversible():
    a = _square(k=0.7, x0=[[0.1, 0, 0], [3, 0.2, 0], [0, 3, 0.3], [3, 3, 0]])
    a.set_momenta(np.ones((len(a), 3)))
    b = leapfrog(a, 1, False)
    c = leapfrog(b, -1, False)
    assert np.allclose(c.positions, a.positions, rtol=0, atol=1e-10)
    assert np.allclose(c.get_momenta(), a.get_momenta(), rtol=0, atol=1e-10)


def test_dynamics_rolls_downhill_both_ways():
    """test_sim/test_dynamics.py: from an expanded configuration at rest,
    dynamics forward or backward in time lowers the potential energy."""
    for step in (1.0, -1.0):
        ideal = np.array([[-1.5, -1.5, 0], [1.5, -1.5, 0], [-1.5, 1.5, 0],
                          [1.5, 1.5, 0]])
        a = Atoms('Au4', ideal * 1.02)
        a.set_calculator(_Well(k=2.0, x0=ideal))
        a.set_velocities(np.zeros((4, 3)))
        start = a.get_potential_energy()
        traj = classical_dynamics(a, step, 5)
        assert len(traj) == 6
        assert min(t.get_potential_energy() for t in traj) < start


def test_leapfrog_conserves_energy():
    a = _square(k=1.0, x0=np.zeros((4, 3)))
    a.set_momenta(np.full((len(a), 3), 5.0))
    e0 = a.get_total_energy()
    x = a
    es = []
    for _ in range(400):
        x = leapfrog(x, 0.5, False)
        es.append(x.get_total_energy())
    # velocity Verlet on a harmonic well: bounded O((w h)^2) oscillation
    assert np.max(np.abs(np.array(es) - e0)) <= 1e-3 * e0


def test_hmc_is_reproducible_and_moves():
    """The deprecated fixed-length HMC (unit-mass kicks, as the reference's
    hmc.py): light atoms so that proposals are accepted."""
    def run(seed):
        a = Atoms('H4', [[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0]])
        a.set_calculator(_Well(k=0.2, x0=np.zeros((4, 3))))
        rng = np.random.RandomState(seed)
        traj, acc, acc_num = run_hmc(a, 30, 0.05, 5, 0.9, 0.0, 0.65, 1.02,
                                     0.98, 0.001, 0.5, temp=1, rng=rng)
        return traj, acc
    t1, acc1 = run(3)
    t2, acc2 = run(3)
    assert len(t1) > 1 and any(acc1)
    assert acc1 == acc2
    assert np.array_equal(t1[-1].positions, t2[-1].positions)
    assert not np.array_equal(t1[-1].positions, t1[0].positions)


def test_nuts_is_reproducible_and_samples():
    def run(seed):
        a = _square(k=0.05, x0=np.zeros((4, 3)))
        ens = NUTSCanonicalEnsemble(a, temperature=300, escape_level=6,
                                    seed=seed)
        traj, meta = ens.run(6)
        return traj, meta, ens
    t1, m1, e1 = run(11)
    t2, m2, _ = run(11)
    assert len(t1) >= 2 and m1['accepted_samples'] == len(t1) - 1
    assert len(t1) == len(t2)
    for x, y in zip(t1, t2):
        assert np.array_equal(x.positions, y.positions)
    assert np.all(np.isfinite(e1.pe)) and np.isfinite(e1.step_size)
    assert e1.step_size > 0
    # a different seed takes a different path
    t3, _, _ = run(12)
    assert not all(np.array_equal(x.positions, y.positions)
                   for x, y in zip(t1[1:], t3[1:])) or len(t3) != len(t1)


def _gcmc_run(mu, steps, seed, resolution=None):
    from pyiid_gb300.sim.gcmc import GrandCanonicalEnsemble
    np.random.seed(seed)  # the reference draws symbols and tests from it
    a = Atoms('Au3', [[1, 1, 1], [2, 1, 1], [1, 2, 1]])
    a.set_cell([6.0, 6.0, 6.0])
    a.set_calculator(_Well(k=0.1))
    ens = GrandCanonicalEnsemble(a, {'Au': mu}, temperature=1000, seed=seed,
                                 resolution=resolution)
    assert ens._engine is None  # a plain calculator: the reference path
    ens.run(steps)
    return ens


def test_gcmc_reference_path_bookkeeping_and_reproducibility():
    for resolution in (None, 0.5):
        e1 = _gcmc_run(0.5, 60, 7, resolution)
        e2 = _gcmc_run(0.5, 60, 7, resolution)
        m = e1.metadata
        assert sum(m[k] for k in ('accepted_additions', 'rejected_additions',
                                  'accepted_removals',
                                  'rejected_removals')) == 60
        n_acc = m['accepted_additions'] + m['accepted_removals']
        assert len(e1.traj) == 1 + n_acc
        assert len(e1.traj[-1]) == 3 + m['accepted_additions'] - \
            m['accepted_removals']
        assert len(e1.traj) == len(e2.traj)
        for x, y in zip(e1.traj, e2.traj):
            assert np.array_equal(x.positions, y.positions)
        # inserted atoms land inside the cell
        assert np.all(e1.traj[-1].positions >= 0)
        assert np.all(e1.traj[-1].positions <= 6.0 + 1e-12)


def test_gcmc_chemical_potential_decides_the_extremes():
    # mu >> any energy change: every insertion accepted; mu << : every
    # removal accepted while more than one atom is left
    e = _gcmc_run(1e6, 40, 3)
    assert e.metadata['rejected_additions'] == 0
    assert e.metadata['accepted_additions'] > 0
    e = _gcmc_run(-1e6, 40, 3)
    assert e.metadata['accepted_additions'] == 0
    assert len(e.traj[-1]) == 1


def _springs(x, k=0.3, r0=2.8):
    """E = k/2 sum_{i<j} (r_ij - r0)^2 and its forces (translation
    invariant, so the samplers' centring does not change it)."""
    d = x[:, None, :] - x[None, :, :]
    r = np.sqrt((d * d).sum(-1))
    np.fill_diagonal(r, 1.0)
    dr = r - r0
    np.fill_diagonal(dr, 0.0)
    e = 0.25 * k * float((dr * dr).sum())
    f = -k * ((dr / r)[:, :, None] * d).sum(1)
    return e, f


class _Springs(Calculator):
    implemented_properties = ['energy', 'forces']

    def calculate(self, atoms=None, properties=['energy'],
                  system_changes=()):
        Calculator.calculate(self, atoms, properties, system_changes)
        e, f = _springs(self.atoms.positions)
        self.results['energy'] = e
        self.results['forces'] = f


def test_spring_forces_are_minus_the_gradient():
    x = np.random.default_rng(0).normal(size=(5, 3)) * 2
    e, f = _springs(x)
    h = 1e-6
    for i, c in ((0, 0), (3, 2), (4, 1)):
        xp, xm = x.copy(), x.copy()
        xp[i, c] += h
        xm[i, c] -= h
        assert abs((_springs(xp)[0] - _springs(xm)[0]) / (2 * h)
                   + f[i, c]) < 1e-6


def _spring_batch(x):
    """(U [B], F [B, N, 3]) of _springs for a torch batch of positions."""
    import torch
    out = [_springs(xi.numpy()) for xi in x]
    return (torch.tensor([e for e, _ in out], dtype=torch.float64),
            torch.as_tensor(np.stack([f for _, f in out])))


def _spring_starts(n_chains):
    base = np.array([[0, 0, 0], [2.8, 0, 0], [0, 2.8, 0], [0, 0, 2.8],
                     [2.0, 2.0, 2.0]], float)
    rng = np.random.default_rng(4)
    return [base + rng.normal(scale=0.1, size=base.shape)
            for _ in range(n_chains)]


def test_nuts_engine_grows_the_tree_as_the_recursive_algorithm():
    """The engine's leaf-by-leaf tree (one batch of chains, lock step, under
    masks) against an independent recursive NUTS (oracle/nuts_np.py,
    Hoffman and Gelman's BuildTree) reading the same keyed random tables:
    every chain's samples, acceptance count, leapfrog count and adapted
    step size agree."""
    import torch
    from oracle.nuts_np import RecursiveNUTS
    from pyiid_gb300.nuts import NUTSEngine
    starts = _spring_starts(4)
    seeds = [5, 6, 7, 8]
    masses = Atoms('Au5').get_masses()
    iters = 7
    eng = NUTSEngine(_spring_batch, np.stack(starts), masses, 300.0, seeds,
                     escape_level=5, device='cpu')
    eng.run(iters)
    for c, (x0, seed) in enumerate(zip(starts, seeds)):
        ref = RecursiveNUTS(_springs, x0, masses, 300.0, seed, 5)
        # the first-step searches agree
        assert abs(float(eng.mu[c]) - ref.mu) <= 1e-12 * abs(ref.mu)
        for _ in range(iters):
            ref.iterate()
        assert int(eng.accepted[c]) == ref.accepted > 0
        assert int(eng.leapfrogs[c]) == ref.leapfrogs
        assert len(eng.samples[c]) == len(ref.samples)
        for a, b in zip(eng.samples[c], ref.samples):
            assert np.allclose(a.numpy(), b, rtol=0, atol=1e-12)
        assert abs(float(eng.step[c]) - ref.eps) <= 1e-12 * ref.eps


def test_sequential_nuts_equals_a_chain_of_a_batch():
    """The drop-in NUTSCanonicalEnsemble (one chain, the attached
    calculator) and chain c of a batched engine with seed c make the same
    decisions sample for sample; the batch evaluates all chains together
    (one evaluation per tick, twice with the re-centred point)."""
    from pyiid_gb300.nuts import NUTSEngine
    starts = _spring_starts(3)
    seeds = [5, 6, 7]
    n_steps = 6
    seq = []
    for x0, seed in zip(starts, seeds):
        a = Atoms('Au5', x0)
        a.set_calculator(_Springs())
        ens = NUTSCanonicalEnsemble(a, temperature=300, escape_level=5,
                                    seed=seed)
        traj, meta = ens.run(n_steps)
        seq.append((traj, meta, ens.step_size))
    eng = NUTSEngine(_spring_batch, np.stack(starts),
                     Atoms('Au5').get_masses(), 300.0, seeds,
                     escape_level=5, device='cpu')
    eng.run(n_steps)
    for c, (traj, meta, step) in enumerate(seq):
        assert meta['accepted_samples'] > 0
        assert int(eng.accepted[c]) == meta['accepted_samples']
        assert int(eng.samples_total[c]) == meta['samples_total']
        assert len(eng.samples[c]) == len(traj) - 1
        for x, t in zip(eng.samples[c], traj[1:]):
            assert np.allclose(x.numpy(), t.positions, rtol=0, atol=1e-9)
        assert abs(float(eng.step[c]) - step) <= 1e-12 * step
    total = sum(int(v) for v in eng.leapfrogs)
    assert eng.evaluations < 2 * total + 64


class _Voxelled(_Well):
    """A well that also reports voxel and atomwise energies (as the spring
    calculators do), to check MultiCalc's sums of them."""

    def calculate_voxel_energy(self, atoms, resolution):
        c = np.diagonal(atoms.get_cell())
        return np.full(tuple(int(x / resolution) for x in c), self.k)

    def calculate_atomwise_energy(self, atoms):
        return np.full(len(atoms), 2.0 * self.k)


def test_multicalc_sums_energies_forces_and_maps():
    """pyiid/calc/multi_calc.py:8-125: the composite calculator's energy,
    forces, voxel and atomwise energies are the sums over its calculators
    (those without voxel / atomwise methods contribute nothing), and the
    atoms keep the composite calculator attached."""
    from pyiid_gb300.calc.multi_calc import MultiCalc
    x0 = [[0.2, 0, 0], [3, 0.1, 0], [0, 3, 0.3], [3, 3, 0]]
    parts = [_Well(k=0.7, x0=x0), _Well(k=0.2), _Voxelled(k=0.5)]
    a = _square()
    a.set_cell([4.0, 4.0, 4.0])
    want_e, want_f = 0.0, np.zeros((4, 3))
    for c in parts:
        b = _square()
        b.set_calculator(c)
        want_e += b.get_potential_energy()
        want_f += b.get_forces()
    mc = MultiCalc(calc_list=parts)
    a.set_calculator(mc)
    assert abs(a.get_potential_energy() - want_e) <= 1e-12 * abs(want_e)
    assert np.allclose(a.get_forces(), want_f, rtol=0, atol=1e-12)
    assert a.calc is mc
    vox = mc.calculate_voxel_energy(a, 0.5)
    assert vox.shape == (8, 8, 8) and np.all(vox == 0.5)
    assert np.all(mc.calculate_atomwise_energy(a) == 1.0)
    # energies follow the positions (the sub-calculators' caches too)
    a.positions[0, 0] += 0.5
    b = _square()
    b.positions[0, 0] += 0.5
    e2 = 0.0
    for c in parts:
        b.set_calculator(c)
        e2 += b.get_potential_energy()
    assert abs(a.get_potential_energy() - e2) <= 1e-12 * abs(e2)
