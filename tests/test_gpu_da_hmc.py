"""Delayed-acceptance HMC on the GPU: the surrogate-force kernels against
the FP64 oracle, and the sampler's device iteration.

* neighbour lists (pyiid_neighbor_list) against a brute-force search;
* descriptors from the lists equal to the oracle's (BF16 rounding);
* surrogate energies and forces (pyiid_surrogate_forces: BF16 tensor-core
  MLP forward and input gradient, pair forces) against the oracle fed the
  same BF16 roundings (oracle/mlp_np.py, whose force formula is pinned by
  central differences on the CPU);
* a DelayedAcceptanceHMC iteration captured in a CUDA graph equals the eager
  iteration bit for bit, and the exact second stage decides as the exact
  energies say.
"""
import ctypes

import numpy as np
import pytest

from oracle import mlp_np as M
from pyiid_gb300 import structures as S

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _batch():
    p1 = S.displaced(S.fcc_nearest(4.08, 140), 0.1, 1)
    p2 = S.displaced(S.fcc_nearest(4.08, 70), 0.1, 2)
    return np.concatenate([p1, p2]).astype(np.float32), np.array(
        [0, 140, 210], np.int32)


def _lists(sur, pos_t, off, r_list, max_nb):
    import torch
    n = pos_t.shape[0]
    nbr = torch.full((n, max_nb), -1, dtype=torch.int32, device='cuda')
    cnt = torch.zeros(n, dtype=torch.int32, device='cuda')
    offp = np.ascontiguousarray(off, np.int32)
    sur.ctx.call('pyiid_neighbor_list', ctypes.c_void_p(pos_t.data_ptr()),
                 offp.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                 len(off) - 1, ctypes.c_float(r_list), max_nb,
                 ctypes.c_void_p(nbr.data_ptr()),
                 ctypes.c_void_p(cnt.data_ptr()))
    torch.cuda.synchronize()
    return nbr, cnt


def test_neighbour_lists_match_brute_force():
    import torch
    from pyiid_gb300.surrogate import RBFMLPSurrogate
    sur = RBFMLPSurrogate()
    pos, off = _batch()
    pt = torch.as_tensor(pos, device='cuda')
    nbr, cnt = _lists(sur, pt, off, 6.5, 128)
    nbr, cnt = nbr.cpu().numpy(), cnt.cpu().numpy()
    for c in range(2):
        a0, a1 = off[c], off[c + 1]
        d = pos[a0:a1, None].astype(np.float32) - pos[None, a0:a1]
        r2 = (d * d).sum(-1)
        for a in range(a0, a1):
            want = [a0 + b for b in np.nonzero(r2[a - a0] < 6.5 ** 2)[0]
                    if a0 + b != a]
            assert cnt[a] == len(want)
            assert list(nbr[a, :cnt[a]]) == want
    # a list shorter than the neighbours reports the overflow
    _, cnt2 = _lists(sur, pt, off, 6.5, 8)
    assert np.array_equal(cnt2.cpu().numpy(), cnt)


def _weights(sur, seed):
    import torch
    g = torch.Generator(device='cpu').manual_seed(seed)
    for k in ('b1', 'b2', 'w3', 'b3'):
        sur.params[k].copy_(torch.randn(sur.params[k].shape, generator=g)
                            .to('cuda') * 0.1)


@pytest.mark.parametrize('centres,hidden,mlp', [(32, 128, 0), (32, 128, 1),
                                               (32, 128, 2), (16, 64, 0)],
                         ids=['fused-32-128-mma.sync', 'fused-32-128-tcgen05',
                              'fused-32-128-tcgen05-two-tiles', 'gemm-16-64'])
def test_surrogate_energy_and_forces_match_oracle(centres, hidden, mlp):
    """The 32-128-128 net runs one fused kernel (register-resident mma.sync
    variant 0, tensor-memory tcgen05 variants 1 and 2), other sizes the
    GEMM chain; all against the oracle."""
    import torch
    from pyiid_gb300._native import context
    from pyiid_gb300.surrogate import DelayedAcceptanceHMC, RBFMLPSurrogate
    ctx = context()
    old_mlp = ctx.get_variant('mlp')
    ctx.set_variant('mlp', mlp)
    try:
        _check_surrogate(centres, hidden)
    finally:
        ctx.set_variant('mlp', old_mlp)


def _surrogate_call(sur, pos, off, max_nb=256):
    """Energies and forces through the sampler's call path, on a stand-in
    holding only what it reads; returns (e, f, da)."""
    import torch
    from pyiid_gb300.surrogate import DelayedAcceptanceHMC
    pt = torch.as_tensor(pos, device='cuda')
    nbr, cnt = _lists(sur, pt, off, sur.rc + 1.0, max_nb)
    da = DelayedAcceptanceHMC.__new__(DelayedAcceptanceHMC)
    da.sur, da.B = sur, len(off) - 1
    da.off, da._offp = off, off.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    da.nbr, da.cnt, da.max_nb = nbr, cnt, max_nb
    da.feat = torch.empty((len(pos), sur.C), dtype=torch.bfloat16,
                          device='cuda')
    da.es = torch.empty(len(off) - 1, dtype=torch.float64, device='cuda')
    da.fs = torch.empty((len(pos), 3), dtype=torch.float32, device='cuda')

    class _P:
        conv = 3.0
    da.pot = _P()
    w1b, b1, w2b = sur._effective()
    p = sur.params
    da.w = {'w1b': w1b, 'b1': b1, 'w2b': w2b, 'b2': p['b2'], 'w3': p['w3'],
            'b3': p['b3']}
    e, f = da.surrogate(pt)
    torch.cuda.synchronize()
    return e, f, da


def test_tensor_memory_mlps_equal_mma_sync_over_many_tiles():
    """48 x 1,000-atom configurations (375 tiles of 128 atoms, more than the
    304 tile slots of the two-tile kernel on 152 SMs, so slots take several
    tiles and some a partial one): both tcgen05 forms against the mma.sync
    form, which the oracle test pins at small size.  Same BF16 roundings of
    the activations; the per-atom output sums differ in order only."""
    from pyiid_gb300._native import context
    from pyiid_gb300.surrogate import RBFMLPSurrogate
    sur = RBFMLPSurrogate(seed=5)
    _weights(sur, 6)
    ref = S.fcc_nearest(4.08, 1000)
    pos = np.concatenate([S.displaced(ref, 0.05, 100 + c)
                          for c in range(48)]).astype(np.float32)
    off = (np.arange(49) * 1000).astype(np.int32)
    ctx = context()
    old = ctx.get_variant('mlp')
    out = {}
    try:
        for v in (0, 1, 2):
            ctx.set_variant('mlp', v)
            e, f, _ = _surrogate_call(sur, pos, off)
            out[v] = (e.cpu().numpy(), f.cpu().numpy())
    finally:
        ctx.set_variant('mlp', old)
    for v in (1, 2):
        assert rel(out[v][0], out[0][0]) < 1e-6, (v, rel(out[v][0], out[0][0]))
        assert rel(out[v][1], out[0][1]) < 1e-5, (v, rel(out[v][1], out[0][1]))


@pytest.mark.parametrize('mlp', [2, 0], ids=['tcgen05-two-tiles', 'mma.sync'])
def test_surrogate_matches_oracle_at_1000_atoms(mlp):
    """The delayed-acceptance configuration's size: two displaced 1,000-atom
    fcc Au particles, energies and forces of the 32-128-128 network against
    the FP64 oracle with the GPU's BF16 roundings mirrored."""
    from pyiid_gb300._native import context
    from pyiid_gb300.surrogate import RBFMLPSurrogate
    sur = RBFMLPSurrogate(seed=5)
    _weights(sur, 6)
    ref = S.fcc_nearest(4.08, 1000)
    pos = np.concatenate([S.displaced(ref, 0.05, 7 + c)
                          for c in range(2)]).astype(np.float32)
    off = np.array([0, 1000, 2000], np.int32)
    ctx = context()
    old = ctx.get_variant('mlp')
    ctx.set_variant('mlp', mlp)
    try:
        e, f, _ = _surrogate_call(sur, pos, off)
    finally:
        ctx.set_variant('mlp', old)
    pc = {k: v.cpu().numpy().astype(np.float64) for k, v in sur.params.items()}
    eo, fo = M.surrogate_energy_forces(pos, off, sur.C, sur.rc, sur.sigma,
                                       pc['w1'], pc['b1'], pc['w2'], pc['b2'],
                                       pc['w3'], pc['b3'], scale=3.0)
    assert rel(e.cpu().numpy(), 3.0 * eo) < 1e-3
    assert rel(f.cpu().numpy(), fo) < 3e-2, rel(f.cpu().numpy(), fo)


def _check_surrogate(centres, hidden):
    from pyiid_gb300.surrogate import RBFMLPSurrogate
    sur = RBFMLPSurrogate(n_centres=centres, n_hidden=hidden, seed=5)
    _weights(sur, 6)
    pos, off = _batch()
    e, f, da = _surrogate_call(sur, pos, off)
    p = sur.params
    # descriptors from the lists are the all-pairs kernel's (summed in
    # another order, so equal to BF16 rounding)
    want = M.rbf_features(pos, off, sur.C, sur.rc, sur.sigma)
    assert rel(da.feat.float().cpu().numpy(), want) < 5e-3
    assert rel(sur.features(pos, off).float().cpu().numpy(), want) < 5e-3
    pc = {k: v.cpu().numpy().astype(np.float64) for k, v in p.items()}
    eo, fo = M.surrogate_energy_forces(pos, off, sur.C, sur.rc, sur.sigma,
                                       pc['w1'], pc['b1'], pc['w2'], pc['b2'],
                                       pc['w3'], pc['b3'], scale=3.0)
    assert rel(e.cpu().numpy(), 3.0 * eo) < 1e-3
    assert rel(f.cpu().numpy(), fo) < 3e-2, rel(f.cpu().numpy(), fo)


def _au_potential(n_chains, n_atoms=200):
    import torch
    from pyiid_gb300 import debye
    from pyiid_gb300.sampling import PDFPotential, experiment_grids
    from pyiid_gb300.scatter_factors import species_tables
    exp, qb, nb, rg = experiment_grids({'rmax': 20.0})
    ref = S.fcc_nearest(4.08, n_atoms).astype(np.float32)
    sp, tab, _ = species_tables([79] * n_atoms, qb, nb)
    gobs = debye.pdf(debye.fq(ref, sp, tab, qb), qb, exp['rstep'], rg,
                     exp['qmin']).cpu().numpy()
    pot = PDFPotential([79] * n_atoms, gobs, {'rmax': 20.0}, conv=100.0,
                       n_configs=n_chains)
    xs = np.stack([S.displaced(ref, 0.05, 40 + c) for c in range(n_chains)])
    return pot, xs


def test_graph_iteration_equals_eager():
    from pyiid_gb300.surrogate import DelayedAcceptanceHMC, RBFMLPSurrogate
    pot, xs = _au_potential(4)
    runs = []
    for graph in (False, True):
        sur = RBFMLPSurrogate(seed=1)
        da = DelayedAcceptanceHMC(pot, sur, xs, temperature=300, dt=5e-3,
                                  n_steps=5, seed=9, graph=graph)
        da.step(4)
        runs.append((da.x.cpu().numpy(), da.E.cpu().numpy(),
                     da.accepted.cpu().numpy(), da.stage1.cpu().numpy()))
        da.check()
    for a, b in zip(*runs):
        assert np.array_equal(a, b)


def test_second_stage_uses_exact_energies():
    """After every iteration the chains' energies are the exact potential of
    their positions (stage 2 decided on exact energies), and accepted
    moves moved the atoms."""
    import torch
    from pyiid_gb300.surrogate import DelayedAcceptanceHMC, RBFMLPSurrogate
    pot, xs = _au_potential(6)
    sur = RBFMLPSurrogate(seed=2)
    da = DelayedAcceptanceHMC(pot, sur, xs, temperature=300, dt=5e-3,
                              n_steps=5, seed=3)
    x0 = da.x.clone()
    da.step(5)
    e = pot.evaluate(da.x, want_grad=False)[0]
    assert torch.allclose(e, da.E, rtol=0, atol=1e-12)
    moved = (da.x - x0).reshape(6, -1).abs().amax(1) > 0
    assert torch.equal(moved, da.accepted > 0)
    assert bool((da.accepted <= da.stage1).all())


def test_trained_network_beats_untrained_at_1000_atoms():
    """1,000-atom Au, E = 100 Rw at 300 K, 10 leapfrog steps of dt = 1e-3
    driven by the surrogate's forces, 16 chains: a network pre-trained on
    exact Rw of displaced particles leaves a smaller exact second-stage log
    ratio (rms, in kT) and accepts more proposals than the untrained
    network, on the same chains and random streams."""
    import torch
    from pyiid_gb300 import debye
    from pyiid_gb300.sampling import PDFPotential, experiment_grids
    from pyiid_gb300.scatter_factors import species_tables
    from pyiid_gb300.surrogate import DelayedAcceptanceHMC, RBFMLPSurrogate
    n, chains, iters = 1000, 16, 8
    exp, qb, nb, rg = experiment_grids(None)
    ref = S.fcc_nearest(4.08, n).astype(np.float32)
    sp, tab, _ = species_tables([79] * n, qb, nb)
    gobs = debye.pdf(debye.fq(ref, sp, tab, qb), qb, exp['rstep'], rg,
                     exp['qmin']).cpu().numpy()
    pot = PDFPotential([79] * n, gobs, None, conv=100.0, n_configs=chains)
    start = np.stack([S.displaced(ref, 0.05, 4 + c) for c in range(chains)])
    # pre-training set: exact Rw of displaced particles (0.01-0.2 A)
    pool = 96
    sig = np.random.default_rng(5).uniform(0.01, 0.2, pool)
    xs = np.stack([S.displaced(ref, s, 5000 + i) for i, s in enumerate(sig)])
    ppot = PDFPotential([79] * n, gobs, None, n_configs=pool)
    rw = ppot.evaluate(torch.as_tensor(xs.reshape(-1, 3), device='cuda'),
                       want_grad=False)[0].clone()
    trained = RBFMLPSurrogate(seed=0, lr=3e-3)
    fb = trained.features(xs.reshape(-1, 3), ppot.offsets)
    for _ in range(200):
        trained.train_step(fb, ppot.offsets, rw)
    res = {}
    for name, sur in (('trained', trained), ('untrained',
                                             RBFMLPSurrogate(seed=0))):
        da = DelayedAcceptanceHMC(pot, sur, start, temperature=300.0,
                                  dt=1e-3, n_steps=10, seed=4, graph=True)
        da.step(iters)
        rms = float((da.sum_dhs_err / (iters * chains)).sqrt()) / da.kT
        res[name] = (int(da.accepted.sum().item()), rms)
        da.check()
    (acc_t, rms_t), (acc_u, rms_u) = res['trained'], res['untrained']
    assert rms_t < 0.8 * rms_u, res
    assert acc_t > acc_u, res
