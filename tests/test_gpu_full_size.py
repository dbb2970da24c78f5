"""The 20,000-atom Pt particle timed by bench.py (fcc a = 3.92 A, the
20,000 sites nearest the origin, displacements sigma 0.02 A with seed 2;
Q 0.5-30 step 0.02, 1,475 bins returned) at full size through the one-pass
call: F(Q) on 17 sampled bins and the complete gradient rows of 16 seeded
atoms against FP64 sums of the C oracle, and size-independent properties of
the whole [20000, 3, 1500] output.  Tolerances as everywhere (norm-wise
relative): F(Q) <= 1e-5, gradient <= 1e-4."""
import numpy as np
import pytest

from oracle import debye_c as C
from oracle import debye_np as O
from pyiid_gb300 import structures as S
from pyiid_gb300.scatter_factors import species_tables

pytestmark = pytest.mark.gpu

TOL_F = 1e-5
TOL_G = 1e-4


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_pt20000_one_pass_against_fp64_samples():
    from pyiid_gb300 import debye
    pos = S.displaced(S.fcc_nearest(3.92, 20000), 0.02, 2)
    qbin, nb, kb = 0.02, 1500, 25
    sp, tab, _ = species_tables([78] * len(pos), qbin, nb)
    f, g = debye.fq_grad(pos, sp, tab, qbin, k_begin=kb)
    f, g = f.cpu().numpy(), g.cpu().numpy()
    assert f.shape == (nb,) and g.shape == (len(pos), 3, nb)

    # FP64 oracle: pair sums on every 92nd returned bin, full rows of 16 atoms
    na = O.normalization(tab[sp])
    bins = np.arange(kb, nb, 92, dtype=np.int32)
    want_f = 2 * C.pair_sums(pos, sp, tab, qbin, bins) / na[bins]
    rows = np.sort(np.random.default_rng(20000).choice(len(pos), 16,
                                                       replace=False))
    # the reference's convention: -dS/dx / na (= -1/2 dF/dx)
    want_g = -C.grad_rows(pos, sp, tab, qbin, rows.astype(np.int32)) / na

    # whole output: bins below qmin are zero, everything finite, and the
    # rows sum to zero (F depends on differences of positions only)
    assert np.all(f[:kb] == 0) and np.all(g[:, :, :kb] == 0)
    assert np.isfinite(f).all() and np.isfinite(g).all()
    total = g.sum(axis=0, dtype=np.float64)
    assert np.linalg.norm(total) <= 1e-4 * np.linalg.norm(g), \
        np.linalg.norm(total) / np.linalg.norm(g)

    assert rel(f[bins], want_f) <= TOL_F, rel(f[bins], want_f)
    for i, a in enumerate(rows):
        e = rel(g[a, :, kb:], want_g[i, :, kb:])
        assert e <= TOL_G, (int(a), e)
