"""The delayed-acceptance rule leaves the exact target unchanged (CPU).

1D toy: exact energy E(x) = x^2/2 (kT = 1, target N(0, 1)); a deliberately
wrong surrogate E~(x) = 0.6 x^2 + 0.3 x screens random-walk proposals.  The
two-stage chain must sample N(0, 1); the surrogate alone would sample
N(-0.25, 0.83).
"""
import numpy as np

from pyiid_gb300.surrogate import da_stage1, da_stage2


def test_delayed_acceptance_targets_exact_distribution():
    rng = np.random.default_rng(0)
    E = lambda x: 0.5 * x * x          # noqa: E731
    Es = lambda x: 0.6 * x * x + 0.3 * x  # noqa: E731
    n_chains, n_steps = 256, 4000
    x = rng.normal(size=n_chains)
    samples = []
    exact_calls = 0
    for t in range(n_steps):
        xp = x + rng.normal(0, 1.0, n_chains)
        ds = Es(xp) - Es(x)
        p1 = da_stage1(np.log(rng.random(n_chains)), ds, 1.0)
        exact_calls += int(p1.sum())
        de = E(xp) - E(x)
        p2 = da_stage2(np.log(rng.random(n_chains)), de, ds, 1.0)
        acc = p1 & p2
        x = np.where(acc, xp, x)
        if t > 500:
            samples.append(x.copy())
    s = np.concatenate(samples)
    assert abs(s.mean()) < 0.02, s.mean()
    assert abs(s.var() - 1.0) < 0.03, s.var()
    # the screen saved exact evaluations
    assert exact_calls < 0.9 * n_chains * n_steps


def test_delayed_acceptance_hmc_keeps_the_exact_target():
    """DelayedAcceptanceHMC's iteration (surrogate-driven leapfrog, two-stage
    acceptance) on a harmonic well with a deliberately wrong surrogate:
    exact energy k/2 |x|^2 per atom (k = 2 kT, so each coordinate has
    variance 1/2), surrogate k~ = 0.5 k shifted by 0.3 A along x.  The chains
    must sample the exact Gaussian (mean 0, variance kT/k), not the
    surrogate's (mean 0.3, variance kT/k~)."""
    import torch
    from pyiid_gb300.atoms import kB
    from pyiid_gb300.surrogate import DelayedAcceptanceHMC

    T = 300.0
    kT = kB * T
    k, ks = 2 * kT, kT

    class Pot:
        device = torch.device('cpu')
        n_configs = 4000
        offsets = np.arange(n_configs + 1, dtype=np.int32)
        n_total = n_configs
        masses = np.full(n_configs, 1.0)
        conv = 1.0

        def config_index(self):
            return torch.arange(self.n_configs)

        def evaluate(self, x, want_grad=True, out=None):
            e = 0.5 * k * (x.double() ** 2).sum(1)
            return e, None

    class Sur:
        rc, C, H = 1.0, 2, 2

    class Toy(DelayedAcceptanceHMC):
        def __init__(self):
            self.pot, self.sur = Pot(), Sur()
            self.kT, self.dt, self.n_steps = kT, 0.9, 3
            self.B = self.N = Pot.n_configs
            self.m = torch.ones((self.N, 1))
            self.cfg = torch.arange(self.N)
            self.gen = torch.Generator().manual_seed(3)
            self.x = torch.zeros((self.N, 3))
            self.E = self.pot.evaluate(self.x)[0]
            self.accepted = torch.zeros(self.B, dtype=torch.int64)
            self.stage1 = torch.zeros(self.B, dtype=torch.int64)
            self.max_cnt = torch.zeros((), dtype=torch.int32)
            self.cnt = torch.zeros(self.N, dtype=torch.int32)
            self.max_disp = torch.zeros(())
            self.sum_dhs_err = torch.zeros((), dtype=torch.float64)
            self.sum_work_err = torch.zeros((), dtype=torch.float64)
            self.buf_size, self.buf_n, self.proposed = 0, 0, 0
            self.graph = None

        def _neighbours(self, x):
            pass

        def surrogate(self, x):
            d = x.double() - torch.tensor([0.3, 0.0, 0.0],
                                          dtype=torch.float64)
            return 0.5 * ks * (d ** 2).sum(1), (-ks * d).float()

    toy = Toy()
    xs = []
    for t in range(300):
        toy.step()
        if t >= 50:
            xs.append(toy.x.double().clone())
    x = torch.cat(xs).numpy()
    acc = toy.acceptance()
    assert 0.2 < acc['accepted'].mean() < 0.95
    assert abs(x.mean()) < 0.01, x.mean(0)
    assert abs(x[:, 0].mean()) < 0.015
    # exact variance kT/k = 0.5 (the surrogate alone would give 1.0)
    assert abs(x.var(0) - kT / k).max() < 0.02, x.var(0)
    # the exact stage corrected what the surrogate stage let through
    assert acc['accepted'].mean() < acc['stage1'].mean() - 0.1
