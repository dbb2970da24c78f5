"""Learned surrogate and delayed acceptance on the GPU.

Checks the radial-basis descriptors and the BF16 tensor-core MLP (forward
and backward) against the FP64 NumPy oracle fed the same BF16-rounded
inputs, that online training fits exact Rw values, and that delayed
acceptance with the trained network needs fewer exact evaluations per
accepted move than without it.
"""
import numpy as np
import pytest

from oracle import mlp_np as M
from pyiid_gb300 import structures as S

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_rbf_features_match_oracle():
    import torch
    from pyiid_gb300.surrogate import RBFMLPSurrogate
    sur = RBFMLPSurrogate()
    p1 = S.displaced(S.fcc_nearest(4.08, 120), 0.1, 1)
    p2 = S.displaced(S.fcc_nearest(4.08, 60), 0.1, 2)
    pos = np.concatenate([p1, p2])
    off = np.array([0, 120, 180])
    fb, ff = sur.features(pos, off, want_f32=True)
    want = M.rbf_features(pos, off, 32, 8.0, sur.sigma)
    assert rel(ff.cpu().numpy(), want) < 1e-5
    assert rel(fb.float().cpu().numpy(), want) < 5e-3   # BF16 rounding


def test_mlp_forward_backward_match_oracle():
    import torch
    from pyiid_gb300.surrogate import RBFMLPSurrogate
    sur = RBFMLPSurrogate(seed=3)
    for k in ('b1', 'b2', 'w3', 'b3'):
        sur.params[k].normal_(0, 0.1)
    pos = np.concatenate([S.displaced(S.fcc_nearest(4.08, 150), 0.1, s)
                          for s in range(3)])
    off = np.array([0, 150, 300, 450])
    fb = sur.features(pos, off)
    e = sur.forward(fb, off).cpu().numpy()
    de = torch.tensor([0.7, -1.3, 0.4], dtype=torch.float64, device='cuda')
    g = {k: v.cpu().numpy() for k, v in sur.backward(de).items()}
    p = {k: v.cpu().numpy().astype(np.float64) for k, v in sur.params.items()}
    X = fb.float().cpu().numpy().astype(np.float64)
    w1b, w2b = M.bf16(p['w1']), M.bf16(p['w2'])
    eo, cache = M.mlp_forward(X, off, w1b, p['b1'], w2b, p['b2'], p['w3'],
                              p['b3'])
    assert rel(e, eo) < 1e-3, (e, eo)
    go = M.mlp_backward(X, off, cache, w2b, p['w3'], de.cpu().numpy())
    for k in go:
        assert rel(g[k], go[k]) < 2e-2, (k, rel(g[k], go[k]))


def _training_set(n_cfg=96, n=200, seed=0):
    import torch
    from pyiid_gb300.sampling import PDFPotential
    from pyiid_gb300 import debye
    from pyiid_gb300.scatter_factors import species_tables
    pot0 = None
    ref = S.fcc_nearest(4.08, n).astype(np.float32)
    exp = {'rmax': 20.0}
    from pyiid_gb300.sampling import experiment_grids
    e, qb, nb, rg = experiment_grids(exp)
    sp, tab, _ = species_tables([79] * n, qb, nb)
    gobs = debye.pdf(debye.fq(ref, sp, tab, qb), qb, e['rstep'], rg,
                     e['qmin']).cpu().numpy()
    rng = np.random.default_rng(seed)
    sig = rng.uniform(0.01, 0.25, n_cfg)
    xs = np.stack([S.displaced(ref, s, 1000 + i) for i, s in enumerate(sig)])
    pot = PDFPotential([79] * n, gobs, exp, n_configs=n_cfg)
    rw = pot.evaluate(torch.as_tensor(xs.reshape(-1, 3), device='cuda'),
                      want_grad=False)[0]
    return pot, gobs, exp, ref, xs, rw


def test_surrogate_training_fits_exact_rw():
    from pyiid_gb300.surrogate import RBFMLPSurrogate
    pot, gobs, exp, ref, xs, rw = _training_set()
    sur = RBFMLPSurrogate(seed=0, lr=3e-3)
    off = pot.offsets
    fb = sur.features(xs.reshape(-1, 3), off)
    losses = [sur.train_step(fb, off, rw) for _ in range(400)]
    assert losses[-1] < 0.05 * losses[0], (losses[0], losses[-1])
    # generalises to held-out configurations of the same family
    pot2, _, _, _, xs2, rw2 = _training_set(n_cfg=32, seed=9)
    pred = sur.predict(xs2.reshape(-1, 3), pot2.offsets)
    r2 = 1 - ((pred - rw2) ** 2).sum() / ((rw2 - rw2.mean()) ** 2).sum()
    assert r2.item() > 0.8, r2.item()


def test_delayed_acceptance_gains_from_the_trained_network():
    """Exact evaluations per accepted move: trained surrogate < untrained."""
    import torch
    from pyiid_gb300.sampling import PDFPotential
    from pyiid_gb300.surrogate import (RBFMLPSurrogate, DelayedAcceptanceMH,
                                       ExactSingleAtomMH)
    pot, gobs, exp, ref, xs, rw = _training_set()
    trained = RBFMLPSurrogate(seed=0, lr=3e-3)
    fb = trained.features(xs.reshape(-1, 3), pot.offsets)
    for _ in range(400):
        trained.train_step(fb, pot.offsets, rw)
    untrained = RBFMLPSurrogate(seed=1)
    untrained.fit_normalisation(fb)
    chains = 16
    start = np.stack([S.displaced(ref, 0.05, 50 + c) for c in range(chains)])
    cpot = PDFPotential([79] * 200, gobs, exp, conv=100.0, n_configs=chains)
    res = {}
    for name, sur in (('trained', trained), ('untrained', untrained)):
        da = DelayedAcceptanceMH(cpot, sur, start, temperature=300, step=0.1,
                                 seed=5)
        for _ in range(40):
            da.iterate()
        res[name] = (da.accepted, da.exact_evals, da.proposed)
    ex = ExactSingleAtomMH(cpot, start, temperature=300, step=0.1, seed=5)
    for _ in range(40):
        ex.iterate()
    acc_t, ev_t, _ = res['trained']
    acc_u, ev_u, _ = res['untrained']
    assert acc_t > 0 and ex.accepted > 0
    # the trained screen spends fewer exact evaluations per accepted move
    assert ev_t / acc_t < ev_u / max(acc_u, 1)
    assert ev_t / acc_t < ex.exact_evals / ex.accepted
