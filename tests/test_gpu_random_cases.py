"""Seeded random cases through every pair-kernel entry point against the
FP64 oracle: atom counts that leave partial tiles, one to three species,
odd bin counts, odd and even k_begin (the packed kernels start at an even
bin), batches of uneven configurations, and small configurations whose
tiles J are split over several CTAs.  Tolerances as everywhere: F(Q)
1e-5, gradients 1e-4 (norm-wise relative)."""
import numpy as np
import pytest

from oracle import debye_np as O
from pyiid_gb300 import structures as S
from pyiid_gb300.scatter_factors import species_tables

pytestmark = pytest.mark.gpu

TOL_F, TOL_G = 1e-5, 1e-4


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.fixture(scope='module')
def D():
    from pyiid_gb300 import debye
    return debye


def case(seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(2, 160))
    elements = [79, 78, 46][:int(rng.integers(1, 4))]
    nums = list(rng.choice(elements, n))
    pos = S.random_cube(n, float(rng.uniform(6.0, 16.0)), seed)
    qbin = float(rng.choice([0.05, 0.1, 0.0756865]))
    nb = int(rng.integers(60, 420))
    kb = int(rng.integers(0, 9))
    return pos, nums, qbin, nb, kb


@pytest.mark.parametrize('seed', range(12))
def test_random_single_configuration(D, seed):
    pos, nums, qbin, nb, kb = case(seed)
    sp, tab, _ = species_tables(nums, qbin, nb)
    want_f = O.fq(pos, tab[sp], qbin)
    want_g = O.grad_fq(pos, tab[sp], qbin)
    f = D.fq(pos, sp, tab, qbin, k_begin=kb).cpu().numpy()
    g = D.grad_fq(pos, sp, tab, qbin, k_begin=kb).cpu().numpy()
    f1, g1 = (t.cpu().numpy() for t in D.fq_grad(pos, sp, tab, qbin, kb))
    for ff in (f, f1):
        assert np.all(ff[:kb] == 0)
        assert rel(ff[kb:], want_f[kb:]) <= TOL_F, (seed, rel(ff[kb:], want_f[kb:]))
    for gg in (g, g1):
        assert np.all(gg[:, :, :kb] == 0)
        assert rel(gg[:, :, kb:], want_g[:, :, kb:]) <= TOL_G, seed


@pytest.mark.parametrize('seed', range(4))
def test_random_batches(D, seed):
    rng = np.random.default_rng(100 + seed)
    sizes = rng.integers(1, 90, int(rng.integers(2, 7)))
    qbin, nb, kb = 0.05, int(rng.integers(80, 300)), int(rng.integers(0, 5))
    elements = [79, 78]
    nums = [list(rng.choice(elements, n)) for n in sizes]
    flat = [z for c in nums for z in c]
    sp, tab, _ = species_tables(flat, qbin, nb)
    pos = np.concatenate([S.random_cube(n, 10.0, 100 + seed + i)
                          for i, n in enumerate(sizes)])
    offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int32)
    got = D.batch_fq(pos, sp, offsets, tab, qbin, kb).cpu().numpy()
    for c in range(len(sizes)):
        p = pos[offsets[c]:offsets[c + 1]]
        s = sp[offsets[c]:offsets[c + 1]]
        want = O.fq(p, tab[s], qbin)
        assert np.all(got[c, :kb] == 0)
        if sizes[c] > 1:
            assert rel(got[c, kb:], want[kb:]) <= TOL_F, (seed, c)
        else:
            assert np.all(got[c] == 0)
