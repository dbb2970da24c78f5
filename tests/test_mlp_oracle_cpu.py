"""The surrogate's FP64 oracle (oracle/mlp_np.py) pinned on the CPU before
the GPU kernels are checked against it: bfloat16 rounding known answers,
the backward pass against central differences of the forward pass, and the
radial-basis descriptors of a two-atom case in closed form."""
import numpy as np
import pytest

from oracle import mlp_np as M


def test_bf16_rounding_known_answers():
    # representable values stay; halfway cases go to the even neighbour
    x = np.array([1.0, -2.5, 0.0, 2.0 ** 127, 2.0 ** -126], np.float32)
    assert np.array_equal(M.bf16(x), x.astype(np.float64))
    one = 1.0
    half_ulp = 2.0 ** -8           # bf16 keeps 7 fraction bits at 1.0
    assert M.bf16(np.float32(one + half_ulp)) == one                 # tie, even
    assert M.bf16(np.float32(one + 3 * half_ulp)) == one + 4 * half_ulp  # tie, even
    assert M.bf16(np.float32(one + 1.5 * half_ulp)) == one + 2 * half_ulp
    assert M.bf16(np.float32(one + 0.5 * half_ulp)) == one
    assert M.bf16(np.float32(-(one + 1.5 * half_ulp))) == -(one + 2 * half_ulp)


def _net(rng, n_in=6, n_h=5):
    return dict(w1=rng.normal(size=(n_in, n_h)) * 0.5,
                b1=rng.normal(size=n_h) * 0.1,
                w2=rng.normal(size=(n_h, n_h)) * 0.5,
                b2=rng.normal(size=n_h) * 0.1,
                w3=rng.normal(size=n_h) * 0.5,
                b3=rng.normal(size=1) * 0.1)


def test_backward_matches_central_differences(monkeypatch):
    """With the BF16 rounding of the hidden layer switched off (identity),
    mlp_backward is the exact gradient of sum_c de_c e_c."""
    monkeypatch.setattr(M, 'bf16', lambda x: np.asarray(x, np.float64))
    rng = np.random.default_rng(1)
    X = rng.normal(size=(7, 6))
    offsets = np.array([0, 3, 7])
    de = np.array([0.7, -1.3])
    net = _net(rng)

    def loss(n):
        e, _ = M.mlp_forward(X, offsets, n['w1'], n['b1'], n['w2'], n['b2'],
                             n['w3'], n['b3'])
        return float(de @ e)

    _, cache = M.mlp_forward(X, offsets, net['w1'], net['b1'], net['w2'],
                             net['b2'], net['w3'], net['b3'])
    g = M.mlp_backward(X, offsets, cache, net['w2'], net['w3'], de)
    h = 1e-6
    for name, arr in net.items():
        for idx in list(np.ndindex(arr.shape))[:6]:
            p = {k: v.copy() for k, v in net.items()}
            m = {k: v.copy() for k, v in net.items()}
            p[name][idx] += h
            m[name][idx] -= h
            fd = (loss(p) - loss(m)) / (2 * h)
            assert abs(fd - g[name][idx]) <= 1e-6 * max(1.0, abs(fd)), \
                (name, idx, fd, g[name][idx])


@pytest.mark.parametrize('d', [1.0, 3.7, 7.9, 8.5])
def test_two_atom_descriptors_in_closed_form(d):
    rc, sigma, n_c = 8.0, 0.5, 32
    pos = np.array([[0, 0, 0], [d, 0, 0], [50, 0, 0]], float)
    f = M.rbf_features(pos, np.array([0, 3]), n_c, rc, sigma)
    mu = np.arange(n_c) * rc / (n_c - 1)
    fc = 0.5 * (1 + np.cos(np.pi * d / rc)) if d < rc else 0.0
    want = np.exp(-(d - mu) ** 2 / (2 * sigma ** 2)) * fc
    assert np.allclose(f[0], want, rtol=1e-12, atol=1e-300)
    assert np.allclose(f[1], want, rtol=1e-12, atol=1e-300)
    assert np.all(f[2] == 0)   # no neighbour within the cutoff


def test_surrogate_forces_are_minus_the_energy_gradient():
    """The force formula of the surrogate oracle (descriptor derivatives of
    both atoms of every pair, back-propagated MLP) against central
    differences of its energy, all in FP64 (no BF16 rounding)."""
    from oracle import mlp_np as M
    rng = np.random.default_rng(5)
    C, H, rc = 8, 16, 5.0
    sig = rc / (C - 1)
    w1 = rng.normal(size=(C, H)) / np.sqrt(C)
    w2 = rng.normal(size=(H, H)) / np.sqrt(H)
    b1, b2 = rng.normal(size=H) * .1, rng.normal(size=H) * .1
    w3, b3 = rng.normal(size=H) * .3, np.array([0.2])
    pos = rng.uniform(0, 6, (12, 3))
    off = np.array([0, 7, 12])
    e, f = M.surrogate_energy_forces(pos, off, C, rc, sig, w1, b1, w2, b2,
                                     w3, b3, scale=2.5, rounded=False)
    h = 1e-6
    for a, c in ((0, 0), (3, 1), (8, 2), (11, 0)):
        xp, xm = pos.copy(), pos.copy()
        xp[a, c] += h
        xm[a, c] -= h
        ep = M.surrogate_energy_forces(xp, off, C, rc, sig, w1, b1, w2, b2,
                                       w3, b3, rounded=False)[0].sum()
        em = M.surrogate_energy_forces(xm, off, C, rc, sig, w1, b1, w2, b2,
                                       w3, b3, rounded=False)[0].sum()
        assert abs(-2.5 * (ep - em) / (2 * h) - f[a, c]) <= 1e-6 * max(
            1.0, abs(f[a, c]))
