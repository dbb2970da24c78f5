"""One-pass F(Q) + gradient (pyiid_fq_grad) against the FP64 oracle and
against the separate F(Q) and gradient calls.

Tolerances as the separate calls' (norm-wise relative to the oracle):
F(Q) <= 1e-5, gradient <= 1e-4.  The fused F(Q) takes every unordered pair
once (tiles J >= I, the diagonal tile's two orders at weight 1/2), sums
groups of 4 J tiles in FP32 and beyond that with compensation, so it agrees
with pyiid_fq to rounding, not bitwise.
"""
import numpy as np
import pytest

from oracle import debye_np as O
from pyiid_gb300 import structures as S
from pyiid_gb300.scatter_factors import species_tables

pytestmark = pytest.mark.gpu

TOL_F = 1e-5
TOL_G = 1e-4


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.fixture(scope='module')
def D():
    from pyiid_gb300 import debye
    return debye


def alloy(n, seed, edge):
    nums = list(np.random.default_rng(seed).choice([78, 79], n))
    return S.random_cube(n, edge, seed), nums


CASES = [
    ('au2', np.array([[0, 0, 0], [3, 0, 0]], np.float32), [79, 79]),
    ('rand77', S.random_cube(77, 14.0, 2), [79] * 77),
    ('alloy50', *alloy(50, 3, 12.0)),
    # more than 4 J tiles of one species (the FP32 groups are flushed
    # inside a species block) and a species change after a partial group
    ('fcc249', S.displaced(S.fcc_sphere(4.08, 10.0), 0.05, 1), [79] * 249),
    ('alloy300', *alloy(300, 5, 18.0)),
    ('three_species', S.random_cube(170, 16.0, 7),
     list(np.random.default_rng(7).choice([46, 78, 79], 170))),
]


@pytest.mark.parametrize('name,pos,numbers', CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize('qbin,nbins,kb', [(0.05, 500, 2), (0.1, 250, 3)])
def test_fq_grad_matches_oracle(D, name, pos, numbers, qbin, nbins, kb):
    sp, tab, _ = species_tables(numbers, qbin, nbins)
    f, g = D.fq_grad(pos, sp, tab, qbin, k_begin=kb)
    f, g = f.cpu().numpy(), g.cpu().numpy()
    want_f = O.fq(pos, tab[sp], qbin)
    want_g = O.grad_fq(pos, tab[sp], qbin)
    assert np.all(f[:kb] == 0) and np.all(g[:, :, :kb] == 0)
    assert rel(f[kb:], want_f[kb:]) <= TOL_F, rel(f[kb:], want_f[kb:])
    assert rel(g[:, :, kb:], want_g[:, :, kb:]) <= TOL_G


def test_fq_grad_agrees_with_the_separate_calls(D):
    pos, nums = alloy(260, 11, 17.0)
    qbin, nb, kb = 0.05, 500, 2
    sp, tab, _ = species_tables(nums, qbin, nb)
    f, g = D.fq_grad(pos, sp, tab, qbin, k_begin=kb)
    f1 = D.fq(pos, sp, tab, qbin, k_begin=kb)
    g1 = D.grad_fq(pos, sp, tab, qbin, k_begin=kb)
    assert rel(f.cpu().numpy(), f1.cpu().numpy()) <= 1e-6
    assert rel(g.cpu().numpy(), g1.cpu().numpy()) <= 1e-6


def test_every_fq_grad_variant_matches_oracle(D):
    from pyiid_gb300 import autotune
    from pyiid_gb300._native import context
    pos, nums = alloy(140, 21, 14.0)
    qbin, nb, kb = 0.05, 500, 3
    sp, tab, _ = species_tables(nums, qbin, nb)
    want_f = O.fq(pos, tab[sp], qbin)
    want_g = O.grad_fq(pos, tab[sp], qbin)
    ctx = context()
    old = ctx.get_variant('fq_grad')
    try:
        for idx, info in autotune.variants('fq_grad'):
            ctx.set_variant('fq_grad', idx)
            f, g = D.fq_grad(pos, sp, tab, qbin, k_begin=kb)
            f, g = f.cpu().numpy(), g.cpu().numpy()
            assert rel(f[kb:], want_f[kb:]) <= TOL_F, (idx, info)
            assert rel(g[:, :, kb:], want_g[:, :, kb:]) <= TOL_G, (idx, info)
    finally:
        ctx.set_variant('fq_grad', old)


def test_fq_grad_edge_cases(D):
    qbin, nb = 0.1, 250
    sp1, tab1, _ = species_tables([79], qbin, nb)
    for n in (0, 1):
        f, g = D.fq_grad(np.zeros((n, 3), np.float32), sp1[:n], tab1, qbin)
        assert f.shape == (nb,) and np.all(f.cpu().numpy() == 0)
        assert g.shape == (n, 3, nb) and np.all(g.cpu().numpy() == 0)
    # coincident atoms: F is 0 in every bin, their gradient rows are 0
    pos = np.array([[0, 0, 0], [0, 0, 0], [3, 0, 0]], np.float32)
    sp3, tab3, _ = species_tables([79] * 3, qbin, nb)
    f, g = D.fq_grad(pos, sp3, tab3, qbin)
    assert np.all(f.cpu().numpy() == 0)
    g = g.cpu().numpy()
    want = O.grad_fq(pos, tab3[sp3], qbin)
    assert np.all(g[:2] == 0)
    assert rel(g[2], want[2]) <= TOL_G
    # k_begin at and beyond the grid: everything 0
    pos2 = S.random_cube(10, 5.0, 9)
    sp, tab, _ = species_tables([79] * 10, qbin, nb)
    for kb in (nb, nb + 5):
        f, g = D.fq_grad(pos2, sp, tab, qbin, k_begin=kb)
        assert np.all(f.cpu().numpy() == 0) and np.all(g.cpu().numpy() == 0)


def test_fq_grad_repeatable_bitwise(D):
    pos, nums = alloy(200, 4, 15.0)
    sp, tab, _ = species_tables(nums, 0.05, 500)
    a = [t.cpu().numpy() for t in D.fq_grad(pos, sp, tab, 0.05)]
    b = [t.cpu().numpy() for t in D.fq_grad(pos, sp, tab, 0.05)]
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_fq_grad_rejects_wrong_output_sizes(D):
    import torch
    from pyiid_gb300._native import NativeError
    pos = S.random_cube(8, 5.0, 1)
    sp, tab, _ = species_tables([79] * 8, 0.1, 50)
    with pytest.raises(NativeError):
        D.fq_grad(pos, sp, tab, 0.1,
                  out_fq=torch.empty(49, dtype=torch.float32, device='cuda'))
    with pytest.raises(NativeError):
        D.fq_grad(pos, sp, tab, 0.1,
                  out_grad=torch.empty((8, 3, 49), dtype=torch.float32,
                                       device='cuda'))


def test_fq_grad_large_particle_sampled(D):
    """2000-atom fcc Pt on the Q 0.5-30 step 0.02 grid: F(Q) on every 16th
    bin and the full gradient rows of 12 seeded atoms against FP64 sums."""
    pos = S.displaced(S.fcc_nearest(3.92, 2000), 0.02, 2)
    qbin, nb, kb = 0.02, 1500, 25
    sp, tab, _ = species_tables([78] * len(pos), qbin, nb)
    f, g = D.fq_grad(pos, sp, tab, qbin, k_begin=kb)
    f, g = f.cpu().numpy(), g.cpu().numpy()
    q = pos.astype(np.float32).astype(np.float64)
    fa = tab[0].astype(np.float64)
    na = O.normalization(tab[sp])
    idx = np.arange(kb, nb, 16)
    Q = idx * qbin
    s = np.zeros(len(idx))
    for i0 in range(1, len(q)):
        d = np.sqrt(((q[i0] - q[:i0]) ** 2).sum(1))
        s += (np.sin(Q[None] * d[:, None]) / d[:, None]).sum(0)
    want_f = 2 * s * fa[idx] ** 2 / na[idx]
    assert rel(f[idx], want_f) <= TOL_F, rel(f[idx], want_f)
    Qa = np.arange(nb) * qbin
    rows = np.random.default_rng(12).choice(len(q), 12, replace=False)
    for a in rows:
        d = q[a] - np.delete(q, a, axis=0)            # [N-1, 3]
        r = np.sqrt((d * d).sum(1))[:, None]
        qr = Qa[None] * r
        w = (Qa[None] * np.cos(qr) - np.sin(qr) / r) / r ** 2
        want = -(fa * fa)[None, :] * np.einsum('jk,jc->ck', w, d) / na
        assert rel(g[a, :, kb:], want[:, kb:]) <= TOL_G, (a, rel(g[a, :, kb:],
                                                                 want[:, kb:]))


@pytest.mark.parametrize('n_parts', [1, 2, 3, 5])
def test_parts_reassemble_one_configuration(D, n_parts):
    """pyiid_fq_grad_part run for every part on one device: the parts' rows
    partition the atoms and equal the one-call gradient (to rounding: the
    one call splits the tiles J of a configuration this small over several
    CTAs), and the summed raw sums give the one-call F(Q)."""
    import torch
    pos, nums = alloy(300, 8, 18.0)
    qbin, nb, kb = 0.05, 500, 3
    sp, tab, _ = species_tables(nums, qbin, nb)
    f_ref, g_ref = D.fq_grad(pos, sp, tab, qbin, k_begin=kb)
    f_ref, g_ref = f_ref.cpu().numpy(), g_ref.cpu().numpy()
    total = torch.zeros(nb, dtype=torch.float64, device='cuda')
    seen = np.zeros(len(pos), int)
    for p in range(n_parts):
        sums, g, rows = D.fq_grad_part(pos, sp, tab, qbin, kb, p, n_parts)
        total += sums
        seen += rows
        g = g.cpu().numpy()
        assert rel(g[rows], g_ref[rows]) <= 1e-6, p
        assert np.all(g[~rows] == 0), p
    assert np.all(seen == 1)
    f = D.fq_from_sums(sp, tab, kb, total).cpu().numpy()
    assert np.all(f[:kb] == 0)
    assert rel(f, f_ref) <= 1e-6
    assert rel(f[kb:], O.fq(pos, tab[sp], qbin)[kb:]) <= TOL_F


def test_sharded_call_on_one_rank_is_the_one_pass_call(D):
    from pyiid_gb300.distributed import fq_grad_sharded
    pos, nums = alloy(120, 9, 13.0)
    sp, tab, _ = species_tables(nums, 0.1, 250)
    f, g, rows = fq_grad_sharded(pos, sp, tab, 0.1, 2)
    f1, g1 = D.fq_grad(pos, sp, tab, 0.1, k_begin=2)
    assert rows.all()
    assert rel(g.cpu().numpy(), g1.cpu().numpy()) <= 1e-6
    assert rel(f.cpu().numpy(), f1.cpu().numpy()) <= 1e-6


# 150 atoms: J tiles split over CTAs, the combine writes the host rows;
# 7,000 atoms (two species): one part, the pair kernel writes the host rows
# itself and adds the second species block to what it wrote for the first
@pytest.mark.parametrize('n,seed,edge', [(150, 13, 14.0), (7000, 17, 45.0)])
def test_zero_copy_outputs_in_pinned_host_memory(D, n, seed, edge):
    """Pinned CPU outputs are written by the kernel over the host link and
    equal the device outputs bitwise; pageable host memory is rejected
    (Python check and the library's pointer check) before any launch."""
    import ctypes
    import torch
    from pyiid_gb300._native import NativeError, context
    pos, nums = alloy(n, seed, edge)
    qbin, nb, kb = 0.05, 500, 3
    sp, tab, _ = species_tables(nums, qbin, nb)
    f, g = D.fq_grad(pos, sp, tab, qbin, k_begin=kb)
    hf = torch.empty(nb, dtype=torch.float32, pin_memory=True)
    hg = torch.empty((len(pos), 3, nb), dtype=torch.float32, pin_memory=True)
    D.fq_grad(pos, sp, tab, qbin, k_begin=kb, out_fq=hf, out_grad=hg)
    torch.cuda.synchronize()
    assert torch.equal(hf, f.cpu()) and torch.equal(hg, g.cpu())
    with pytest.raises(NativeError):
        D.fq_grad(pos, sp, tab, qbin, out_fq=torch.empty(nb))
    p = D.as_positions(pos)
    page = np.zeros((len(pos), 3, nb), np.float32)
    spi = np.ascontiguousarray(sp, np.int32)
    tabf = np.ascontiguousarray(tab, np.float32)
    with pytest.raises(NativeError):
        context().call('pyiid_fq_grad', ctypes.c_void_p(p.data_ptr()),
                       spi.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                       len(pos), tabf.ctypes.data_as(
                           ctypes.POINTER(ctypes.c_float)),
                       tab.shape[0], nb, qbin, kb,
                       ctypes.c_void_p(f.data_ptr()),
                       ctypes.c_void_p(page.ctypes.data))


@pytest.mark.parametrize('n', [40, 300, 1000])
def test_small_configurations_split_over_ctas(D, n):
    """Configurations too small to fill the GPU split the tiles J of every
    tile I over several CTAs (partial rows added in a fixed order): oracle
    parity, bitwise repeatable, and coincident atoms still give zero rows."""
    pos = S.displaced(S.fcc_nearest(4.08, n), 0.05, n)
    qbin, nb, kb = 0.05, 500, 2
    sp, tab, _ = species_tables([79] * n, qbin, nb)
    f, g = (t.cpu().numpy() for t in D.fq_grad(pos, sp, tab, qbin, kb))
    f2, g2 = (t.cpu().numpy() for t in D.fq_grad(pos, sp, tab, qbin, kb))
    assert np.array_equal(f, f2) and np.array_equal(g, g2)
    if n <= 300:
        assert rel(f[kb:], O.fq(pos, tab[sp], qbin)[kb:]) <= TOL_F
        want = O.grad_fq(pos, tab[sp], qbin)
        assert rel(g[:, :, kb:], want[:, :, kb:]) <= TOL_G
    g1 = D.grad_fq(pos, sp, tab, qbin, kb).cpu().numpy()
    assert rel(g, g1) <= 1e-6
    dup = np.concatenate([pos, pos[:1]])
    sp_d = np.concatenate([sp, sp[:1]])
    _, gd = D.fq_grad(dup, sp_d, tab, qbin, kb)
    gd = gd.cpu().numpy()
    assert np.all(gd[0] == 0) and np.all(gd[-1] == 0)
    gd1 = D.grad_fq(dup, sp_d, tab, qbin, kb).cpu().numpy()
    assert np.all(gd1[0] == 0) and np.all(gd1[-1] == 0)
    assert rel(gd1, gd) <= 1e-6


def _fq_grad_sampled_check(pos, numbers, f, g, qbin, nb, kb, rows=8):
    """F(Q) on every 8th bin and the full gradient rows of a few seeded
    atoms against FP64 sums; zeros below k_begin."""
    sp, tab, _ = species_tables(numbers, qbin, nb)
    q = pos.astype(np.float32).astype(np.float64)
    per = tab[sp].astype(np.float64)
    na = O.normalization(tab[sp])
    assert np.all(f[:kb] == 0) and np.all(g[:, :, :kb] == 0)
    idx = np.arange(kb, nb, 8)
    Q = idx * qbin
    s = np.zeros(len(idx))
    for i0 in range(1, len(q)):
        d = np.sqrt(((q[i0] - q[:i0]) ** 2).sum(1))
        s += ((per[i0, idx][None] * per[:i0][:, idx])
              * np.sin(Q[None] * d[:, None]) / d[:, None]).sum(0)
    want_f = 2 * s / na[idx]
    assert rel(f[idx], want_f) <= TOL_F, rel(f[idx], want_f)
    Qa = np.arange(nb) * qbin
    for a in np.random.default_rng(len(q)).choice(len(q), rows, replace=False):
        others = np.delete(np.arange(len(q)), a)
        d = q[a] - q[others]
        r = np.sqrt((d * d).sum(1))[:, None]
        qr = Qa[None] * r
        w = (per[a][None] * per[others]) * (Qa[None] * np.cos(qr)
                                            - np.sin(qr) / r) / r ** 2
        want = -np.einsum('jk,jc->ck', w, d) / na
        assert rel(g[a, :, kb:], want[:, kb:]) <= TOL_G, a


def test_split_across_sizes_kbegin_species_and_variants(D):
    """Configurations whose tiles J are split over CTAs (parts ordered
    largest first, combined in part order): alternating sizes, odd and zero
    k_begin, three species and every launch variant, each against FP64 sums
    with zeros below k_begin, the gradient-only call within 1e-6, and the
    same input twice bitwise equal."""
    from pyiid_gb300 import autotune
    from pyiid_gb300._native import context
    qbin, nb = 0.05, 500
    fcc = S.displaced(S.fcc_nearest(4.08, 1000), 0.05, 21)
    tri = S.random_cube(300, 18.0, 8)
    tri_n = list(np.random.default_rng(8).choice([46, 78, 79], 300))
    first = None
    for pos, nums, kb in ((fcc, [79] * 1000, 3), (*alloy(64, 9, 11.0), 0),
                          (tri, tri_n, 2), (fcc, [79] * 1000, 3)):
        sp, tab, _ = species_tables(nums, qbin, nb)
        f, g = (t.cpu().numpy() for t in D.fq_grad(pos, sp, tab, qbin, kb))
        _fq_grad_sampled_check(pos, nums, f, g, qbin, nb, kb)
        g1 = D.grad_fq(pos, sp, tab, qbin, kb).cpu().numpy()
        assert rel(g1, g) <= 1e-6
        assert np.all(g1[:, :, :kb] == 0)
        if len(pos) == 1000:
            if first is None:
                first = (f, g)
            else:
                assert np.array_equal(first[0], f)
                assert np.array_equal(first[1], g)
    ctx = context()
    old = ctx.get_variant('fq_grad')
    sp, tab, _ = species_tables(tri_n, qbin, nb)
    try:
        ref = None
        for idx, _ in autotune.variants('fq_grad'):
            ctx.set_variant('fq_grad', idx)
            f, g = (t.cpu().numpy()
                    for t in D.fq_grad(tri, sp, tab, qbin, 3))
            if ref is None:
                _fq_grad_sampled_check(tri, tri_n, f, g, qbin, nb, 3, rows=4)
                ref = (f, g)
            assert rel(f, ref[0]) <= 1e-6 and rel(g, ref[1]) <= 1e-6, idx
            assert np.all(f[:3] == 0) and np.all(g[:, :, :3] == 0)
    finally:
        ctx.set_variant('fq_grad', old)


def test_split_combine_into_an_output_at_an_odd_offset(D):
    """A small configuration (J-split, partial rows combined) written into a
    gradient that starts 4 bytes past a 16-byte boundary: the combine takes
    its scalar path and the result equals the aligned call bitwise."""
    import torch
    pos = S.displaced(S.fcc_nearest(4.08, 300), 0.05, 3)
    qbin, nb, kb = 0.05, 500, 2
    sp, tab, _ = species_tables([79] * 300, qbin, nb)
    f, g = D.fq_grad(pos, sp, tab, qbin, kb)
    big = torch.full((300 * 3 * nb + 4,), float('nan'), device='cuda')
    out = big[1:1 + 300 * 3 * nb].view(300, 3, nb)
    assert out.data_ptr() % 16 == 4
    f2, g2 = D.fq_grad(pos, sp, tab, qbin, kb, out_grad=out)
    assert torch.equal(g2, g) and torch.equal(f2, f)
    assert torch.isnan(big[0]) and torch.isnan(big[-3:]).all()
