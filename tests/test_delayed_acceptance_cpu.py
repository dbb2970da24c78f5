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
