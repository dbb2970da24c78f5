"""Oracle of the single-atom Metropolis path, on the CPU: the Philox
restatement against the published known-answer vectors, the proposal
distribution, and the acceptance rule."""
import numpy as np

from oracle import mh_np


def test_philox_known_answers():
    # Random123 known-answer vectors for Philox4x32-10 (counter, key, output)
    kat = [
        ([0, 0, 0, 0], [0, 0],
         [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
        ([0xffffffff] * 4, [0xffffffff] * 2,
         [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
        ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344],
         [0xa4093822, 0x299f31d0],
         [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]),
    ]
    for ctr, key, out in kat:
        got = mh_np.philox4x32_10(ctr, key)
        assert [int(v) for v in got] == out


def test_philox_vectorised_matches_scalar():
    rng = np.random.default_rng(0)
    ctr = rng.integers(0, 2 ** 32, size=(17, 4), dtype=np.uint64)
    many = mh_np.philox4x32_10(ctr, (123, 456))
    for i in range(len(ctr)):
        assert np.array_equal(many[i], mh_np.philox4x32_10(ctr[i], (123, 456)))


def test_proposal_distribution():
    n, sigma = 37, 0.2
    atoms, ds, lu = [], [], []
    for t in range(4000):
        a, d, logu = mh_np.proposal(99, 3, t, n, sigma)
        atoms.append(a)
        ds.append(d)
        lu.append(logu)
    atoms, ds, lu = np.array(atoms), np.array(ds), np.array(lu)
    assert atoms.min() >= 0 and atoms.max() < n
    counts = np.bincount(atoms, minlength=n)
    # chi^2 of a uniform draw, 36 degrees of freedom (p ~ 1e-4 cut)
    e = len(atoms) / n
    assert ((counts - e) ** 2 / e).sum() < 75
    assert abs(ds.mean()) < 4 * sigma / np.sqrt(ds.size)
    assert abs(ds.std() / sigma - 1) < 0.03
    u = np.exp(lu)
    assert np.all((u > 0) & (u < 1))
    assert abs(u.mean() - 0.5) < 0.02
    # a single-atom configuration always proposes atom 0
    assert all(mh_np.proposal(5, 0, t, 1, 0.1)[0] == 0 for t in range(50))


def test_proposals_depend_on_seed_chain_step_only():
    a = mh_np.proposal(7, 2, 11, 50, 0.1)
    b = mh_np.proposal(7, 2, 11, 50, 0.1)
    c = mh_np.proposal(7, 3, 11, 50, 0.1)
    d = mh_np.proposal(8, 2, 11, 50, 0.1)
    assert a[0] == b[0] and np.array_equal(a[1], b[1]) and a[2] == b[2]
    assert not np.array_equal(a[1], c[1])
    assert not np.array_equal(a[1], d[1])


def test_metropolis_rule():
    assert mh_np.metropolis_accept(np.log(0.5), 1.0, 1.0, 100.0, 0.025)
    assert not mh_np.metropolis_accept(np.log(0.5), 1.1, 1.0, 100.0, 0.025)
    assert mh_np.metropolis_accept(np.log(0.5), 0.9, 1.0, 100.0, 0.025)
    assert not mh_np.metropolis_accept(np.log(0.5), np.nan, 1.0, 1.0, 1.0)


def test_exact_delta_s_is_difference_of_sums():
    rng = np.random.default_rng(1)
    x = rng.normal(size=(12, 3)) * 3
    sp = np.array([0, 1] * 6)
    tab = np.abs(rng.normal(size=(2, 40))) + 1
    d = mh_np.exact_delta_s(x, sp, tab, 0.1, 4, x[4] + [0.1, -0.2, 0.05])
    x2 = x.copy()
    x2[4] += [0.1, -0.2, 0.05]
    # direct restatement: only pairs with atom 4 change
    q = np.arange(40) * 0.1
    ref = np.zeros(40)
    for j in range(12):
        if j == 4:
            continue
        r1 = np.linalg.norm(x2[4] - x[j])
        r0 = np.linalg.norm(x[4] - x[j])
        ff = tab[sp[4]] * tab[sp[j]]
        ref += ff * (np.sin(q * r1) / r1 - np.sin(q * r0) / r0)
    ref[0] = 0.0
    d[0] = 0.0
    assert np.allclose(d, ref, rtol=1e-9, atol=1e-9)
