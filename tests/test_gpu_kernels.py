"""GPU parity of the sm_103a kernels against the FP64 oracle (via the C ABI).

Tolerances (norm-wise relative, ||gpu - oracle|| / ||oracle||):
  F(Q), G(r), potentials      <= 1e-5
  gradients (dF, dG, dRw)     <= 1e-4
The oracle (oracle/debye_np.py) is itself pinned to the reference's own
outputs in tests/test_oracle_golden.py.
"""
import numpy as np
import pytest

from oracle import debye_np as O
from pyiid_gb300.scatter_factors import species_tables, form_factor_array
from pyiid_gb300 import structures as S

pytestmark = pytest.mark.gpu

TOL_F = 1e-5
TOL_G = 1e-4


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.fixture(scope='module')
def D():
    from pyiid_gb300 import debye
    return debye


def per_atom(species, tab):
    return tab[species]


def au_cube(n, seed, edge=10.0):
    return S.random_cube(n, edge, seed)


CASES = [
    ('au2', np.array([[0, 0, 0], [3, 0, 0]], np.float32), [79, 79]),
    ('rand20', S.random_cube(20, 10.0, 1), [79] * 20),
    ('rand77', S.random_cube(77, 14.0, 2), [79] * 77),
    ('alloy50', S.random_cube(50, 12.0, 3),
     list(np.random.default_rng(3).choice([78, 79], 50))),
    ('fcc249', S.displaced(S.fcc_sphere(4.08, 10.0), 0.05, 1), [79] * 249),
]


@pytest.mark.parametrize('name,pos,numbers', CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize('qbin,nbins,kb', [(0.05, 500, 2), (0.1, 250, 0),
                                           (0.0756865, 330, 7)])
def test_fq_matches_oracle(D, name, pos, numbers, qbin, nbins, kb):
    sp, tab, _ = species_tables(numbers, qbin, nbins)
    got = D.fq(pos, sp, tab, qbin, k_begin=kb).cpu().numpy()
    want = O.fq(pos, per_atom(sp, tab), qbin)
    assert np.all(got[:kb] == 0)
    assert rel(got[kb:], want[kb:]) <= TOL_F, rel(got[kb:], want[kb:])


@pytest.mark.parametrize('name,pos,numbers', CASES[:4],
                         ids=[c[0] for c in CASES[:4]])
@pytest.mark.parametrize('qbin,nbins,kb', [(0.05, 500, 2), (0.1, 250, 3)])
def test_grad_fq_matches_oracle(D, name, pos, numbers, qbin, nbins, kb):
    sp, tab, _ = species_tables(numbers, qbin, nbins)
    got = D.grad_fq(pos, sp, tab, qbin, k_begin=kb).cpu().numpy()
    want = O.grad_fq(pos, per_atom(sp, tab), qbin)
    assert np.all(got[:, :, :kb] == 0)
    assert rel(got[:, :, kb:], want[:, :, kb:]) <= TOL_G


def test_fq_large_particle_sampled(D):
    # 2000-atom fcc Pt, Q 0.5-30 step 0.02: compare every 16th bin
    pos = S.displaced(S.fcc_nearest(3.92, 2000), 0.02, 2)
    qbin, nbins, kb = 0.02, 1500, 25
    sp, tab, _ = species_tables([78] * len(pos), qbin, nbins)
    got = D.fq(pos, sp, tab, qbin, k_begin=kb).cpu().numpy()
    idx = np.arange(kb, nbins, 16)
    sub = tab[:, idx]
    # oracle on the sampled bins: pair sums at Q_k = k*qbin
    f = per_atom(sp, tab)
    s = np.zeros(len(idx))
    q = pos.astype(np.float64)
    Q = idx * qbin
    for i0 in range(1, len(q)):
        d = np.sqrt(((q[i0] - q[:i0]) ** 2).sum(1))
        s += (np.sin(Q[None] * d[:, None]) / d[:, None]).sum(0)
    want = 2 * s * sub[0] ** 2 / O.normalization(f)[idx]
    assert rel(got[idx], want) <= TOL_F, rel(got[idx], want)


def test_pdf_matches_oracle(D):
    import torch
    exp = O.update_experiment({'qmin': 0.7, 'rmin': 0.5, 'rmax': 30.0})
    qb = O.pdf_qbin(exp)
    rg = O.r_grid(exp)
    nb = int(np.floor(exp['qmax'] / qb))
    pos = S.displaced(S.fcc_sphere(4.08, 10.0), 0.05, 1)
    sp, tab, _ = species_tables([79] * len(pos), qb, nb)
    f = D.fq(pos, sp, tab, qb)
    g = D.pdf(f, qb, exp['rstep'], rg, exp['qmin']).cpu().numpy()
    want = O.pdf_fft(O.fq(pos, per_atom(sp, tab), qb), exp['rstep'], qb, rg,
                     exp['qmin'])
    assert rel(g, want) <= TOL_F
    # batched rows
    fb = torch.stack([f, 2 * f])
    gb = D.pdf(fb, qb, exp['rstep'], rg, exp['qmin']).cpu().numpy()
    assert rel(gb[1], 2 * want) <= TOL_F


@pytest.mark.parametrize('kind', ['rw', 'chi_sq'])
def test_potential_and_grad_chain_matches_oracle(D, kind):
    import torch
    exp = O.update_experiment({'qmin': 0.6, 'qmax': 22.0, 'qbin': 0.13,
                               'rmin': 0.5, 'rmax': 12.0, 'rstep': 0.05})
    qb = O.pdf_qbin(exp)
    rg = O.r_grid(exp)
    nb = int(np.floor(exp['qmax'] / qb))
    ref = S.random_cube(30, 9.0, 5)
    pos = (ref + np.random.default_rng(6).normal(0, .05, ref.shape)
           ).astype(np.float32)
    sp, tab, _ = species_tables([79] * 30, qb, nb)
    f_ref = O.fq(ref, per_atom(sp, tab), qb)
    gobs = O.pdf_fft(f_ref, exp['rstep'], qb, rg, exp['qmin'])
    f_pos = O.fq(pos, per_atom(sp, tab), qb)
    gcalc = O.pdf_fft(f_pos, exp['rstep'], qb, rg, exp['qmin'])
    want_v = (O.get_rw if kind == 'rw' else O.get_chi_sq)(gobs, gcalc)
    go_t = torch.as_tensor(gobs, device='cuda')
    gc_t = torch.as_tensor(gcalc, device='cuda')
    got = D.potential(go_t, gc_t, kind).cpu().numpy()
    assert abs(got[0] - want_v[0]) <= TOL_F * abs(want_v[0])
    # explicit compat chain: grad_fq -> grad_pdf -> potential_grad
    gq = D.grad_fq(pos, sp, tab, qb)
    gp = D.grad_pdf(gq, qb, exp['rstep'], rg, exp['qmin'])
    gq_o = O.grad_fq(pos, per_atom(sp, tab), qb)
    gp_o = O.grad_pdf(gq_o, exp['rstep'], qb, rg, exp['qmin'])
    assert rel(gp.cpu().numpy(), gp_o) <= TOL_G
    pg = D.potential_grad(gp, gc_t, go_t, kind).cpu().numpy()
    if kind == 'rw':
        want_g = O.get_grad_rw(gp_o, gcalc, gobs, *want_v)
    else:
        want_g = O.get_grad_chi_sq(gp_o, gcalc, gobs, want_v[1])
    assert rel(pg, want_g) <= TOL_G


@pytest.mark.parametrize('kind', ['rw', 'chi_sq'])
def test_batch_adjoint_matches_oracle(D, kind):
    import torch
    exp = O.update_experiment({'qmin': 0.6, 'qmax': 22.0, 'qbin': 0.13,
                               'rmin': 0.5, 'rmax': 14.0, 'rstep': 0.02})
    qb = O.pdf_qbin(exp)
    rg = O.r_grid(exp)
    nb = int(np.floor(exp['qmax'] / qb))
    rng = np.random.default_rng(11)
    sizes = [2, 37, 64, 5, 90]
    ref = S.random_cube(60, 10.0, 12)
    numbers_all, pos_all, offs = [], [], [0]
    for i, n in enumerate(sizes):
        nums = list(rng.choice([78, 79], n)) if i % 2 else [79] * n
        p = S.random_cube(n, 10.0, 100 + i)
        numbers_all += nums
        pos_all.append(p)
        offs.append(offs[-1] + n)
    pos = np.concatenate(pos_all)
    uniq = np.array([78, 79])
    sp = np.searchsorted(uniq, np.asarray(numbers_all)).astype(np.int32)
    tab = np.stack([form_factor_array(z, np.arange(nb) * qb)
                    for z in uniq]).astype(np.float32)
    f_ref = O.fq(ref, np.repeat(tab[1:2], 60, 0), qb)
    gobs = O.pdf_fft(f_ref, exp['rstep'], qb, rg, exp['qmin'])
    out = D.batch_potential_grad(pos, sp, np.array(offs), tab, qb,
                                 exp['rstep'], rg, exp['qmin'],
                                 torch.as_tensor(gobs), kind)
    e = out['energy'].cpu().numpy()
    g = out['grad'].cpu().numpy()
    for i in range(len(sizes)):
        a, b = offs[i], offs[i + 1]
        val, tg = O.true_grad_potential(pos[a:b], tab[sp[a:b]], exp, gobs,
                                        kind)
        assert abs(e[i, 0] - val) <= TOL_F * abs(val) + 1e-12, (i, e[i], val)
        assert rel(g[a:b], tg) <= TOL_G, (i, rel(g[a:b], tg))


def test_edge_cases(D):
    qbin, nb = 0.1, 250
    sp1, tab1, _ = species_tables([79], qbin, nb)
    # one atom and zero atoms: F = 0, gradient = 0 (reference returns zeros)
    assert np.all(D.fq(np.zeros((1, 3), np.float32), sp1, tab1, qbin)
                  .cpu().numpy() == 0)
    assert D.fq(np.zeros((0, 3), np.float32), sp1[:0], tab1, qbin
                ).cpu().numpy().tolist() == [0.0] * nb
    assert np.all(D.grad_fq(np.zeros((1, 3), np.float32), sp1, tab1, qbin)
                  .cpu().numpy() == 0)
    # coincident atoms: the reference's NaN becomes 0 for every bin of F and
    # for the coincident atoms' gradient rows
    pos = np.array([[0, 0, 0], [0, 0, 0], [3, 0, 0]], np.float32)
    sp3, tab3, _ = species_tables([79] * 3, qbin, nb)
    assert np.all(D.fq(pos, sp3, tab3, qbin).cpu().numpy() == 0)
    gq = D.grad_fq(pos, sp3, tab3, qbin).cpu().numpy()
    want = O.grad_fq(pos, tab3[sp3], qbin)
    assert np.all(gq[:2] == 0) and np.all(want[:2] == 0)
    assert rel(gq[2], want[2]) <= TOL_G
    # k_begin beyond the grid: all zero
    pos2 = S.random_cube(10, 5.0, 9)
    sp, tab, _ = species_tables([79] * 10, qbin, nb)
    assert np.all(D.fq(pos2, sp, tab, qbin, k_begin=nb + 5).cpu().numpy() == 0)


def test_bad_arguments_raise(D):
    from pyiid_gb300._native import NativeError
    sp, tab, _ = species_tables([79] * 4, 0.1, 50)
    pos = S.random_cube(4, 5.0, 1)
    with pytest.raises(NativeError):
        D.fq(pos, np.array([0, 1, 0, 0], np.int32), tab, 0.1)  # species >= S
    with pytest.raises(NativeError):
        D.fq(pos, sp, tab, -0.1)


def test_repeatable_bitwise(D):
    pos = S.random_cube(120, 12.0, 4)
    sp, tab, _ = species_tables([79] * 120, 0.05, 500)
    a = D.fq(pos, sp, tab, 0.05).cpu().numpy()
    b = D.fq(pos, sp, tab, 0.05).cpu().numpy()
    assert np.array_equal(a, b)
    ga = D.grad_fq(pos, sp, tab, 0.05).cpu().numpy()
    gb = D.grad_fq(pos, sp, tab, 0.05).cpu().numpy()
    assert np.array_equal(ga, gb)


@pytest.mark.parametrize('kernel', ['fq', 'grad_fq'])
def test_every_launch_variant_matches_oracle(D, kernel):
    """All autotuner variants compute the same (correct) result."""
    from pyiid_gb300 import autotune
    from pyiid_gb300._native import context
    pos = S.random_cube(70, 11.0, 21)
    nums = list(np.random.default_rng(21).choice([78, 79], 70))
    qbin, nb, kb = 0.05, 500, 3
    sp, tab, _ = species_tables(nums, qbin, nb)
    ctx = context()
    old = ctx.get_variant(kernel)
    want_f = O.fq(pos, per_atom(sp, tab), qbin)
    want_g = O.grad_fq(pos, per_atom(sp, tab), qbin)
    try:
        for idx, info in autotune.variants(kernel):
            ctx.set_variant(kernel, idx)
            if kernel == 'fq':
                got = D.fq(pos, sp, tab, qbin, k_begin=kb).cpu().numpy()
                assert rel(got[kb:], want_f[kb:]) <= TOL_F, (idx, info)
            else:
                got = D.grad_fq(pos, sp, tab, qbin, k_begin=kb).cpu().numpy()
                assert rel(got[:, :, kb:], want_g[:, :, kb:]) <= TOL_G, (idx, info)
    finally:
        ctx.set_variant(kernel, old)


def test_autotune_selects_and_caches(D, tmp_path, monkeypatch):
    from pyiid_gb300 import autotune
    from pyiid_gb300._native import context
    monkeypatch.setenv('PYIID_GB300_TUNE_CACHE', str(tmp_path / 't.json'))
    pos = S.random_cube(200, 14.0, 8)
    sp, tab, _ = species_tables([79] * 200, 0.05, 300)
    res = autotune.tune(pos, sp, tab, 0.05, 0, reps=1)
    ctx = context()
    assert ctx.get_variant('fq') == res['fq']['best']
    assert ctx.get_variant('grad_fq') == res['grad_fq']['best']
    ctx.set_variant('fq', 0)
    ctx.set_variant('grad_fq', 0)
    got = autotune.apply_cached(200, 300, 1)
    assert got == {'fq': res['fq']['best'], 'grad_fq': res['grad_fq']['best']}
    ctx.set_variant('fq', DEFAULT_FQ_VARIANT)
    ctx.set_variant('grad_fq', 0)


DEFAULT_FQ_VARIANT = 23


def test_new_context_starts_on_the_group_reduction_variant(D):
    from pyiid_gb300 import autotune
    from pyiid_gb300._native import Context
    ctx = Context(0)
    try:
        assert ctx.get_variant('fq') == DEFAULT_FQ_VARIANT
        assert ctx.get_variant('grad_fq') == 0
        assert ctx.get_variant('adjoint') == 0
    finally:
        ctx.close()
    info = dict(autotune.variants('fq'))[DEFAULT_FQ_VARIANT]
    assert (info['bins_per_thread'], info['pairs_per_thread']) == (56, -3)


def test_batch_fq_uneven_alloys_matches_oracle(D):
    rng = np.random.default_rng(17)
    sizes = [1, 55, 2, 130, 0, 77]
    pos, nums, off = [], [], [0]
    for i, n in enumerate(sizes):
        pos.append(S.random_cube(n, 12.0, 50 + i))
        nums.append(rng.choice([78, 79], n))
        off.append(off[-1] + n)
    pos = np.concatenate(pos)
    allnum = np.concatenate(nums)
    sp, tab, _ = species_tables(allnum, 0.05, 500)
    got = D.batch_fq(pos, sp, np.array(off), tab, 0.05, 2).cpu().numpy()
    for i in range(len(sizes)):
        a, b = off[i], off[i + 1]
        want = O.fq(pos[a:b], tab[sp[a:b]], 0.05) if b - a else np.zeros(500)
        assert np.all(got[i, :2] == 0)
        if b - a < 2:
            assert np.all(got[i] == 0)
        else:
            assert rel(got[i, 2:], want[2:]) <= TOL_F
        single = D.fq(pos[a:b], sp[a:b], tab, 0.05, 2).cpu().numpy()
        assert np.array_equal(single, got[i])


def test_persistent_batch_fq_equals_one_cta_per_unit(D):
    """The persistent F(Q) form (resident CTAs drawing work units from a
    device counter) writes the partial rows the one-CTA-per-unit launch
    writes: an uneven alloy batch is bitwise equal, and equal to the oracle,
    on two calls in a row (the counter is reset per launch)."""
    from pyiid_gb300 import autotune
    from pyiid_gb300._native import context
    rng = np.random.default_rng(29)
    sizes = [int(n) for n in rng.integers(2, 400, 24)]
    pos, nums, off = [], [], [0]
    for i, n in enumerate(sizes):
        pos.append(S.random_cube(n, 14.0, 80 + i))
        nums.append(rng.choice([78, 79], n))
        off.append(off[-1] + n)
    pos = np.concatenate(pos)
    sp, tab, _ = species_tables(np.concatenate(nums), 0.05, 500)
    shapes = {(i['bins_per_thread'], i['pairs_per_thread']): idx
              for idx, i in autotune.variants('fq')}
    ctx = context()
    old = ctx.get_variant('fq')
    try:
        ctx.set_variant('fq', shapes[(56, -3)])
        want = D.batch_fq(pos, sp, np.array(off), tab, 0.05, 2).cpu().numpy()
        ctx.set_variant('fq', shapes[(56, -13)])
        for _ in range(2):
            got = D.batch_fq(pos, sp, np.array(off), tab, 0.05,
                             2).cpu().numpy()
            assert np.array_equal(got, want)
    finally:
        ctx.set_variant('fq', old)
    for i in (0, 7, 23):
        a, b = off[i], off[i + 1]
        o = O.fq(pos[a:b], tab[sp[a:b]], 0.05)
        assert rel(got[i, 2:], o[2:]) <= TOL_F


@pytest.mark.parametrize('variant', [0, 1])
def test_adjoint_variants_match_oracle(D, variant):
    """Symmetric (each pair once) and owner-computes adjoints agree with the
    oracle on a multi-tile alloy batch (diagonal and off-diagonal tiles)."""
    import torch
    from pyiid_gb300._native import context
    exp = O.update_experiment({'qmin': 0.6, 'qmax': 22.0, 'rmin': 0.5,
                               'rmax': 14.0, 'rstep': 0.02})
    qb = O.pdf_qbin(exp)
    rg = O.r_grid(exp)
    nb = int(np.floor(exp['qmax'] / qb))
    sizes = [70, 33, 97]
    rng = np.random.default_rng(5)
    pos = np.concatenate([S.random_cube(n, 11.0, 200 + i)
                          for i, n in enumerate(sizes)])
    nums = rng.choice([78, 79], sum(sizes))
    offs = np.concatenate([[0], np.cumsum(sizes)])
    sp, tab, _ = species_tables(nums, qb, nb)
    gobs = O.pdf_fft(O.fq(S.random_cube(50, 9.0, 3), np.repeat(tab[1:], 50, 0),
                          qb), exp['rstep'], qb, rg, exp['qmin'])
    ctx = context()
    old = ctx.get_variant('adjoint')
    try:
        ctx.set_variant('adjoint', variant)
        out = D.batch_potential_grad(pos, sp, offs, tab, qb, exp['rstep'], rg,
                                     exp['qmin'], torch.as_tensor(gobs))
    finally:
        ctx.set_variant('adjoint', old)
    g = out['grad'].cpu().numpy()
    for i in range(len(sizes)):
        a, b = offs[i], offs[i + 1]
        _, tg = O.true_grad_potential(pos[a:b], tab[sp[a:b]], exp, gobs)
        assert rel(g[a:b], tg) <= TOL_G, (variant, i, rel(g[a:b], tg))
