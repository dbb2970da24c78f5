"""FP64 NumPy restatement of the surrogate (test infrastructure only).

Only tests/ use this module.  It mirrors the definitions documented in
include/pyiid_gb300.h for pyiid_rbf_features / pyiid_mlp_forward /
pyiid_mlp_backward; the checks feed it the same BF16-rounded inputs and
weights the GPU consumes, so the comparison isolates the kernels' arithmetic.
"""
import numpy as np


def bf16(x):
    """Round float32 values to bfloat16 (round to nearest even), as float64."""
    a = np.ascontiguousarray(np.asarray(x, np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def rbf_features(pos, offsets, n_centres, rc, sigma):
    pos = np.asarray(pos, np.float64)
    mu = np.arange(n_centres) * rc / (n_centres - 1)
    out = np.zeros((len(pos), n_centres))
    for c in range(len(offsets) - 1):
        a0, a1 = offsets[c], offsets[c + 1]
        p = pos[a0:a1]
        d = np.sqrt(((p[:, None] - p[None]) ** 2).sum(-1))
        np.fill_diagonal(d, np.inf)
        m = d < rc
        fc = np.where(m, 0.5 * (1 + np.cos(np.pi * np.minimum(d, rc) / rc)), 0)
        g = np.exp(-(d[..., None] - mu) ** 2 / (2 * sigma ** 2)) * fc[..., None]
        out[a0:a1] = g.sum(1)
    return out


def silu(x):
    return x / (1 + np.exp(-x))


def dsilu(x):
    s = 1 / (1 + np.exp(-x))
    return s * (1 + x * (1 - s))


def mlp_forward(X, offsets, w1, b1, w2, b2, w3, b3):
    """X, w1, w2 already BF16-rounded; hidden layer 1 output rounded to BF16
    before layer 2 as the GPU does."""
    z1 = X @ w1 + b1
    h1 = silu(z1)
    h1b = bf16(h1)
    z2 = h1b @ w2 + b2
    h2 = silu(z2)
    y = h2 @ w3 + b3[0]
    e = np.array([y[offsets[c]:offsets[c + 1]].sum()
                  for c in range(len(offsets) - 1)])
    return e, (z1, h1b, z2, h2)


def mlp_backward(X, offsets, cache, w2, w3, de):
    z1, h1b, z2, h2 = cache
    cfg = np.repeat(np.arange(len(offsets) - 1), np.diff(offsets))
    dy = de[cfg]
    g_w3 = h2.T @ dy
    g_b3 = np.array([dy.sum()])
    dz2 = (dy[:, None] * w3[None]) * dsilu(z2)
    g_w2 = h1b.T @ dz2
    g_b2 = dz2.sum(0)
    dz1 = (dz2 @ w2.T) * dsilu(z1)
    g_w1 = X.T @ dz1
    g_b1 = dz1.sum(0)
    return {'w1': g_w1, 'b1': g_b1, 'w2': g_w2, 'b2': g_b2, 'w3': g_w3,
            'b3': g_b3}


def _identity(x):
    return np.asarray(x, np.float64)


def surrogate_energy_forces(pos, offsets, n_centres, rc, sigma, w1, b1, w2,
                            b2, w3, b3, scale=1.0, rounded=True):
    """Energy E_c = sum_a y_a per configuration and forces -scale dE/dx of
    the surrogate (the definition of pyiid_surrogate_forces).

    rounded=True mirrors the GPU's BF16 roundings (descriptors, weights,
    hidden layer 1, and the two back-propagated activations); with
    rounded=False everything is FP64, so the forces are the exact gradient
    of the energy (checked by central differences on the CPU).
    dE/dx_a = sum_b sum_c (g_ac + g_bc) phi_c'(r_ab) (x_a - x_b)/r_ab,
    phi_c = exp(-(r - mu_c)^2 / 2 s^2) fc(r), fc = (1 + cos(pi r/rc))/2."""
    r16 = bf16 if rounded else _identity
    pos = np.asarray(pos, np.float64)
    X = r16(rbf_features(pos, offsets, n_centres, rc, sigma))
    w1r, w2r = r16(w1), r16(w2)
    z1 = X @ w1r + b1
    h1 = r16(silu(z1))
    z2 = h1 @ w2r + b2
    h2 = silu(z2)
    y = h2 @ w3 + b3[0]
    e = np.array([y[offsets[c]:offsets[c + 1]].sum()
                  for c in range(len(offsets) - 1)])
    dz2 = r16(np.broadcast_to(w3, z2.shape) * dsilu(z2))
    dz1 = r16((dz2 @ w2r.T) * dsilu(z1))
    g = dz1 @ w1r.T                        # dE/dfeat [N, C]
    mu = np.arange(n_centres) * rc / (n_centres - 1)
    forces = np.zeros_like(pos)
    for c in range(len(offsets) - 1):
        a0, a1 = offsets[c], offsets[c + 1]
        p = pos[a0:a1]
        d = p[:, None] - p[None]                    # x_a - x_b
        r = np.sqrt((d ** 2).sum(-1))
        np.fill_diagonal(r, np.inf)
        m = r < rc
        rr = np.where(m, r, rc)
        fc = 0.5 * (1 + np.cos(np.pi * rr / rc))
        dfc = -0.5 * np.pi / rc * np.sin(np.pi * rr / rc)
        ex = np.exp(-(rr[..., None] - mu) ** 2 / (2 * sigma ** 2))
        dphi = ex * (dfc[..., None] - fc[..., None] * (rr[..., None] - mu)
                     / sigma ** 2)
        gg = g[a0:a1]
        s = ((gg[:, None, :] + gg[None, :, :]) * dphi).sum(-1)
        s = np.where(m, s / np.where(m, r, 1.0), 0.0)
        forces[a0:a1] = -scale * (s[..., None] * d).sum(1)
    return e, forces
