"""Learned surrogate of Rw and the delayed-acceptance Metropolis sampler.

Surrogate: per-atom Gaussian radial-basis descriptors (32 centres on
[0, 8] A with a cosine cutoff, ``pyiid_rbf_features``) feed a per-atom MLP
32 -> 128 -> 128 -> 1 (SiLU; BF16 tensor-core GEMMs, FP32 accumulate,
``pyiid_mlp_forward`` / ``pyiid_mlp_backward``) whose outputs summed over a
configuration estimate its Rw.  It is trained online on (configuration,
exact Rw) pairs produced by the exact sampler; the parameter update (Adam)
is a handful of elementwise torch ops on the FP32 master copy.

Delayed acceptance (Christen & Fox, J. Comput. Graph. Stat. 14, 2005):
a proposal x' is first accepted with probability
    a1 = min(1, exp(-(E~(x') - E~(x)) / kT))       (surrogate E~ = conv Rw~)
and only then with
    a2 = min(1, exp(-(E(x') - E(x)) / kT + (E~(x') - E~(x)) / kT))
using the exact Debye energy E.  The product kernel satisfies detailed
balance with respect to exp(-E/kT): the chain's target is unchanged and the
exact potential still decides every accepted move.
"""
import ctypes

import numpy as np
import torch

from . import debye
from ._native import NativeError, context
from .atoms import kB

__all__ = ['RBFMLPSurrogate', 'DelayedAcceptanceMH', 'ExactSingleAtomMH',
           'da_stage1', 'da_stage2']


def da_stage1(log_u1, ds, kT):
    """First-stage acceptance on the surrogate energy change ds."""
    return log_u1 < -ds / kT


def da_stage2(log_u2, de, ds, kT):
    """Second-stage acceptance on the exact change de, corrected by the
    surrogate change ds (Christen & Fox 2005, eq. 2)."""
    return log_u2 < -(de - ds) / kT


def _vp(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def _i32(a):
    a = np.ascontiguousarray(np.asarray(a, np.int32))
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


class RBFMLPSurrogate:
    """Sum over atoms of an MLP of radial-basis descriptors.

    Inputs are standardised with statistics of the first training batch,
    folded into the first layer (W1' = W1 / s, b1' = b1 - (mu / s) W1).
    """

    def __init__(self, n_centres=32, r_cut=8.0, sigma=None, n_hidden=128,
                 lr=2e-3, seed=0, device=None):
        self.C = int(n_centres)
        self.rc = float(r_cut)
        self.sigma = float(sigma if sigma is not None else
                           r_cut / (n_centres - 1))
        self.H = int(n_hidden)
        self.dev = torch.device('cuda' if device is None else device)
        g = torch.Generator(device='cpu').manual_seed(int(seed))
        C, H = self.C, self.H
        self.params = {
            'w1': torch.randn(C, H, generator=g) * (1.0 / np.sqrt(C)),
            'b1': torch.zeros(H),
            'w2': torch.randn(H, H, generator=g) * (1.0 / np.sqrt(H)),
            'b2': torch.zeros(H),
            'w3': torch.randn(H, generator=g) * (0.1 / np.sqrt(H)),
            'b3': torch.zeros(1),
        }
        self.params = {k: v.to(self.dev).float().contiguous()
                       for k, v in self.params.items()}
        self.m = {k: torch.zeros_like(v) for k, v in self.params.items()}
        self.v = {k: torch.zeros_like(v) for k, v in self.params.items()}
        self.t = 0
        self.lr = float(lr)
        self.mu = None
        self.scale = None
        self.ctx = context(self.dev.index)

    # ------------------------------------------------------------ kernels
    def features(self, positions, offsets, want_f32=False):
        """BF16 descriptors [N, C] (and FP32 when asked) of packed positions."""
        pos = debye.as_positions(positions)
        off, offp = _i32(offsets)
        n = int(off[-1])
        if off.ndim != 1 or len(off) < 2 or pos.shape[0] < int(off.max()):
            raise NativeError(f'offsets {list(off.shape)} must be [B + 1] '
                              f'and cover at most the {pos.shape[0]} '
                              'positions')
        fb = torch.empty((n, self.C), dtype=torch.bfloat16, device=self.dev)
        ff = (torch.empty((n, self.C), dtype=torch.float32, device=self.dev)
              if want_f32 else None)
        self.ctx.call('pyiid_rbf_features', _vp(pos), offp, len(off) - 1,
                      self.C, ctypes.c_float(self.rc),
                      ctypes.c_float(self.sigma), _vp(fb), _vp(ff))
        return (fb, ff) if want_f32 else fb

    def _effective(self):
        p = self.params
        if self.mu is None:
            w1, b1 = p['w1'], p['b1']
        else:
            w1 = p['w1'] / self.scale[:, None]
            b1 = p['b1'] - (self.mu / self.scale) @ p['w1']
        return (w1.to(torch.bfloat16).contiguous(), b1.contiguous(),
                p['w2'].to(torch.bfloat16).contiguous())

    def forward(self, feat_bf16, offsets):
        """Rw estimates [B] (FP64) for descriptor rows of packed configs."""
        off, offp = _i32(offsets)
        if not (isinstance(feat_bf16, torch.Tensor) and feat_bf16.is_cuda and
                feat_bf16.dtype == torch.bfloat16 and
                feat_bf16.is_contiguous() and
                feat_bf16.numel() == int(off[-1]) * self.C):
            raise NativeError(f'descriptors must be a contiguous bfloat16 '
                              f'CUDA tensor [{int(off[-1])}, {self.C}]')
        w1b, b1, w2b = self._effective()
        self._last = (w1b, b1, w2b)  # keep alive for backward
        e = torch.empty(len(off) - 1, dtype=torch.float64, device=self.dev)
        self._last_b = len(off) - 1
        p = self.params
        self.ctx.call('pyiid_mlp_forward', _vp(feat_bf16), int(off[-1]),
                      self.C, offp, len(off) - 1, _vp(w1b), _vp(b1),
                      _vp(w2b), _vp(p['b2']), _vp(p['w3']), _vp(p['b3']),
                      self.H, _vp(e))
        return e

    def backward(self, d_energy):
        """Parameter gradients (in the standardised parametrisation) of the
        last forward for dL/dE = d_energy [B]."""
        g = {k: torch.empty_like(v) for k, v in self.params.items()}
        de = torch.as_tensor(d_energy).to(device=self.dev,
                                          dtype=torch.float64).contiguous()
        if de.numel() != getattr(self, '_last_b', -1):
            raise NativeError('d_energy must hold one value per configuration '
                              'of the last forward')
        self.ctx.call('pyiid_mlp_backward', _vp(de),
                      _vp(g['w1']), _vp(g['b1']), _vp(g['w2']), _vp(g['b2']),
                      _vp(g['w3']), _vp(g['b3']))
        if self.mu is not None:
            # back through W1' = W1 / s, b1' = b1 - (mu / s) W1
            g['w1'] = g['w1'] / self.scale[:, None] - \
                (self.mu / self.scale)[:, None] * g['b1'][None, :]
        return g

    # ------------------------------------------------------------ training
    def fit_normalisation(self, feat_bf16):
        f = feat_bf16.float()
        self.mu = f.mean(0)
        self.scale = f.std(0).clamp_min(1e-3)

    def predict(self, positions, offsets):
        return self.forward(self.features(positions, offsets), offsets)

    def train_step(self, feat_bf16, offsets, target):
        """One Adam step on the mean squared error; returns the loss."""
        if self.mu is None:
            self.fit_normalisation(feat_bf16)
        e = self.forward(feat_bf16, offsets)
        t = target.to(device=self.dev, dtype=torch.float64)
        r = e - t
        loss = float((r * r).mean().item())
        g = self.backward(2.0 * r / len(r))
        self.t += 1
        b1, b2, eps = 0.9, 0.999, 1e-8
        for k, p in self.params.items():
            gk = g[k].float()
            self.m[k].mul_(b1).add_(gk, alpha=1 - b1)
            self.v[k].mul_(b2).addcmul_(gk, gk, value=1 - b2)
            mh = self.m[k] / (1 - b1 ** self.t)
            vh = self.v[k] / (1 - b2 ** self.t)
            p.sub_(self.lr * mh / (vh.sqrt() + eps))
        return loss


class ExactSingleAtomMH:
    """Lock-step single-atom Metropolis on the exact potential (one move per
    chain per iteration).  The comparator of the delayed-acceptance chain."""

    def __init__(self, pot, positions, temperature=300.0, step=0.1, seed=0):
        self.pot = pot
        self.kT = kB * float(temperature)
        self.step = float(step)
        self.n = int(np.diff(pot.offsets)[0])
        assert np.all(np.diff(pot.offsets) == self.n), 'equal-size chains'
        self.B = pot.n_configs
        self.x = torch.as_tensor(np.asarray(positions, np.float32),
                                 device=pot.device).reshape(self.B, self.n, 3
                                                            ).clone()
        self.gen = torch.Generator(device=pot.device).manual_seed(int(seed))
        self.e = pot.evaluate(self.x.reshape(-1, 3), want_grad=False)[0].clone()
        self.accepted = 0
        self.proposed = 0
        self.exact_evals = 0

    def _propose(self):
        d = self.pot.device
        idx = torch.randint(0, self.n, (self.B,), generator=self.gen, device=d)
        xp = self.x.clone()
        ar = torch.arange(self.B, device=d)
        xp[ar, idx] += self.step * torch.randn((self.B, 3), generator=self.gen,
                                               device=d)
        return xp

    def iterate(self):
        xp = self._propose()
        ep = self.pot.evaluate(xp.reshape(-1, 3), want_grad=False)[0]
        self.exact_evals += self.B
        logu = torch.log(torch.rand(self.B, generator=self.gen,
                                    device=self.x.device, dtype=torch.float64))
        acc = logu < -(ep - self.e) / self.kT
        self.x = torch.where(acc[:, None, None], xp, self.x)
        self.e = torch.where(acc, ep, self.e)
        self.accepted += int(acc.sum().item())
        self.proposed += self.B


class DelayedAcceptanceMH(ExactSingleAtomMH):
    """Single-atom delayed-acceptance Metropolis: surrogate first stage,
    exact Debye second stage (only for proposals that pass the first).

    Online training: every exact second-stage evaluation is stored in a
    replay buffer of (configuration, exact Rw) pairs; every ``train_every``
    iterations the surrogate takes ``train_steps`` Adam steps on a random
    batch of ``train_batch`` buffered pairs.  Surrogate energies of the
    current states are refreshed after training (the first stage compares
    both ends with the same network, as detailed balance requires).
    """

    def __init__(self, pot, surrogate, positions, temperature=300.0, step=0.1,
                 seed=0, train_every=0, train_steps=1, train_batch=64,
                 buffer_size=512):
        super().__init__(pot, positions, temperature, step, seed)
        self.sur = surrogate
        self.off = pot.offsets
        self.es = self._surrogate(self.x)
        self.stage1_passed = 0
        self.train_every = int(train_every)
        self.train_steps = int(train_steps)
        self.train_batch = int(train_batch)
        self.buf_x = torch.empty((int(buffer_size), self.n, 3),
                                 dtype=torch.float32, device=pot.device)
        self.buf_e = torch.empty(int(buffer_size), dtype=torch.float64,
                                 device=pot.device)
        self.buf_n = 0
        self.buf_i = 0
        self.iters = 0

    def _remember(self, xs, rw):
        cap = self.buf_x.shape[0]
        for j in range(xs.shape[0]):
            self.buf_x[self.buf_i] = xs[j]
            self.buf_e[self.buf_i] = rw[j]
            self.buf_i = (self.buf_i + 1) % cap
            self.buf_n = min(self.buf_n + 1, cap)

    def _train(self):
        if self.buf_n < 2:
            return
        b = min(self.train_batch, self.buf_n)
        off = (np.arange(b + 1) * self.n).astype(np.int32)
        for _ in range(self.train_steps):
            idx = torch.randint(0, self.buf_n, (b,), generator=self.gen,
                                device=self.x.device)
            fb = self.sur.features(self.buf_x[idx].reshape(-1, 3), off)
            self.sur.train_step(fb, off, self.buf_e[idx])
        self.es = self._surrogate(self.x)

    def _surrogate(self, x):
        return self.pot.conv * self.sur.predict(x.reshape(-1, 3), self.off)

    def iterate(self):
        self.iters += 1
        if self.train_every and self.iters % self.train_every == 0:
            self._train()
        xp = self._propose()
        esp = self._surrogate(xp)
        d = self.x.device
        u = torch.rand((2, self.B), generator=self.gen, device=d,
                       dtype=torch.float64)
        ds = esp - self.es
        pass1 = da_stage1(torch.log(u[0]), ds, self.kT)
        sel = torch.nonzero(pass1).flatten()
        k = int(sel.numel())
        self.proposed += self.B
        self.stage1_passed += k
        if k == 0:
            return
        # exact energies of the proposals that passed, as one batch of k
        # configurations of the same atoms
        ep = self._exact_subset(xp[sel])
        self.exact_evals += k
        if self.train_every:
            self._remember(xp[sel], ep / self.pot.conv)
        acc = da_stage2(torch.log(u[1][sel]), ep - self.e[sel], ds[sel],
                        self.kT)
        take = sel[acc]
        self.x[take] = xp[take]
        self.e[take] = ep[acc]
        self.es[take] = esp[take]
        self.accepted += int(acc.sum().item())

    def _exact_subset(self, xs):
        from .sampling import PDFPotential
        k = xs.shape[0]
        sub = getattr(self, '_subpots', {}).get(k)
        if sub is None:
            p = self.pot
            sub = PDFPotential.__new__(PDFPotential)
            sub.__dict__.update(p.__dict__)
            sub.n_configs = k
            sub.offsets = (np.arange(k + 1) * self.n).astype(np.int32)
            sub.species = p.species[:k * self.n]
            sub.n_total = k * self.n
            sub.masses = p.masses[:k * self.n]
            sub._out = None
            self._subpots = getattr(self, '_subpots', {})
            self._subpots[k] = sub
        return sub.evaluate(xs.reshape(-1, 3), want_grad=False)[0]


class DelayedAcceptanceHMC:
    """Hamiltonian Monte Carlo whose trajectories follow the surrogate, with
    delayed acceptance (Christen & Fox 2005) on top.

    Every iteration of every chain draws Maxwell-Boltzmann momenta and runs
    ``n_steps`` leapfrog steps of size ``dt`` (BatchedHMC's integrator) with
    the SURROGATE's forces -conv dRw~/dx (``pyiid_surrogate_forces``:
    neighbour-list descriptors, BF16 tensor-core MLP forward and input
    gradient).  Leapfrog on any smooth potential is reversible and volume
    preserving, so the move is a valid Metropolis proposal for the exact
    target exp(-H/kT); it is accepted in two stages:
        stage 1: log u1 < -(H~' - H~)/kT,  H~ = conv Rw~ + K   (surrogate)
        stage 2: log u2 < -[(H' - H) - (H~' - H~)]/kT,  H = conv Rw + K
    with the exact Debye potential (energy only, ``pyiid_batch_potential_grad``
    without gradient) in stage 2, so the chain's target is the exact one
    whatever the surrogate's quality; a poor surrogate costs acceptance, not
    correctness.  The surrogate change H~' - H~ is the kinetic change plus
    the work of the surrogate's forces along the trajectory (trapezoid rule
    over the leapfrog points): for steps of 1e-3 A the BF16 energies
    themselves change by less than their rounding, while the work is smooth.
    Any stage-1 quantity that changes sign when the trajectory is reversed
    keeps delayed acceptance exact (the stage-2 ratio divides it out), and
    the work does.  The exact potential is evaluated once per iteration (at
    the trajectory's end), against once per leapfrog step in BatchedHMC.

    The neighbour lists are built at the start of every trajectory with
    radius r_cut + ``skin``; the largest displacement within a trajectory
    and the largest list length are tracked on the device, and
    :meth:`check` raises when either invalidates the lists.  Exact
    (configuration, Rw) pairs of every stage 2 enter a ring buffer;
    :meth:`train` takes Adam steps on it and copies the new weights into the
    buffers the captured iteration reads.  With ``graph=True`` one iteration
    of all chains is one CUDA graph replay.
    """

    def __init__(self, pot, surrogate, positions, temperature=300.0, dt=1e-3,
                 n_steps=10, seed=0, graph=False, skin=1.0, max_nb=256,
                 buffer_size=2048):
        d = pot.device
        self.pot, self.sur = pot, surrogate
        self.kT = kB * float(temperature)
        self.dt, self.n_steps = float(dt), int(n_steps)
        self.B = pot.n_configs
        self.off, self._offp = _i32(pot.offsets)
        self.N = int(pot.n_total)
        sizes = np.diff(self.off)
        self.n_per = int(sizes[0]) if len(sizes) and np.all(
            sizes == sizes[0]) else None
        self.x = torch.as_tensor(np.asarray(positions, np.float32),
                                 device=d).reshape(-1, 3).clone()
        self.m = torch.as_tensor(pot.masses, dtype=torch.float32,
                                 device=d)[:, None]
        self.cfg = pot.config_index()
        self.gen = torch.Generator(device=d)
        self.gen.manual_seed(int(seed))
        self.max_nb = int(max_nb)
        self.r_list = float(surrogate.rc + skin)
        self.skin = float(skin)
        self.nbr = torch.zeros((self.N, self.max_nb), dtype=torch.int32,
                               device=d)
        self.cnt = torch.zeros(self.N, dtype=torch.int32, device=d)
        self.feat = torch.empty((self.N, surrogate.C), dtype=torch.bfloat16,
                                device=d)
        self.es = torch.empty(self.B, dtype=torch.float64, device=d)
        self.fs = torch.empty((self.N, 3), dtype=torch.float32, device=d)
        C, H = surrogate.C, surrogate.H
        self.w = {'w1b': torch.empty((C, H), dtype=torch.bfloat16, device=d),
                  'b1': torch.empty(H, device=d),
                  'w2b': torch.empty((H, H), dtype=torch.bfloat16, device=d),
                  'b2': torch.empty(H, device=d),
                  'w3': torch.empty(H, device=d),
                  'b3': torch.empty(1, device=d)}
        self.refresh_weights()
        self.E = pot.evaluate(self.x, want_grad=False)[0].clone()
        self.accepted = torch.zeros(self.B, dtype=torch.int64, device=d)
        self.stage1 = torch.zeros(self.B, dtype=torch.int64, device=d)
        self.max_disp = torch.zeros((), dtype=torch.float32, device=d)
        self.max_cnt = torch.zeros((), dtype=torch.int32, device=d)
        self.sum_dhs_err = torch.zeros((), dtype=torch.float64, device=d)
        self.sum_work_err = torch.zeros((), dtype=torch.float64, device=d)
        self.proposed = 0
        # replay buffer of exact (configuration, Rw) pairs (equal-size chains)
        self.buf_size = int(buffer_size) if self.n_per else 0
        if self.buf_size:
            self.buf_x = torch.zeros((self.buf_size, self.n_per, 3),
                                     dtype=torch.float32, device=d)
            self.buf_e = torch.zeros(self.buf_size, dtype=torch.float64,
                                     device=d)
        self.buf_ptr = torch.zeros((), dtype=torch.int64, device=d)
        self.buf_n = 0
        self.graph = None
        if graph:
            self._capture()

    # -------------------------------------------------------------- pieces
    def refresh_weights(self):
        """Copy the surrogate's current (standardisation-folded) weights into
        the buffers the iteration reads."""
        w1b, b1, w2b = self.sur._effective()
        p = self.sur.params
        self.w['w1b'].copy_(w1b)
        self.w['b1'].copy_(b1)
        self.w['w2b'].copy_(w2b)
        self.w['b2'].copy_(p['b2'])
        self.w['w3'].copy_(p['w3'])
        self.w['b3'].copy_(p['b3'])

    def _neighbours(self, x):
        self.sur.ctx.call('pyiid_neighbor_list', _vp(x), self._offp, self.B,
                          ctypes.c_float(self.r_list), self.max_nb,
                          _vp(self.nbr), _vp(self.cnt))

    def surrogate(self, x):
        """(conv Rw~ [B] FP64, forces -conv dRw~/dx [N, 3]) at x, with the
        current neighbour lists."""
        s, w = self.sur, self.w
        conv = float(self.pot.conv)
        s.ctx.call('pyiid_surrogate_forces', _vp(x), self._offp, self.B,
                   _vp(self.nbr), _vp(self.cnt), self.max_nb, s.C,
                   ctypes.c_float(s.rc), ctypes.c_float(s.sigma),
                   _vp(w['w1b']), _vp(w['b1']), _vp(w['w2b']), _vp(w['b2']),
                   _vp(w['w3']), _vp(w['b3']), s.H, ctypes.c_float(conv),
                   _vp(self.es), _vp(self.fs), _vp(self.feat))
        return conv * self.es, self.fs

    def _kinetic(self, p):
        ke_atom = 0.5 * (p.double() ** 2 / self.m.double()).sum(1)
        out = torch.zeros(self.B, dtype=torch.float64, device=p.device)
        return out.index_add_(0, self.cfg, ke_atom)

    def _iteration(self):
        dt = self.dt
        x0 = self.x.clone()
        self._neighbours(x0)
        self.max_cnt.copy_(torch.maximum(self.max_cnt, self.cnt.max()))
        s0, f = self.surrogate(x0)
        s0, f = s0.clone(), f.clone()
        p = torch.randn(x0.shape, generator=self.gen,
                        device=x0.device) * torch.sqrt(self.m * self.kT)
        k0 = self._kinetic(p)
        x = x0
        p = p + 0.5 * dt * f
        disp = torch.zeros((), dtype=torch.float32, device=x0.device)
        work = torch.zeros(self.B, dtype=torch.float64, device=x0.device)
        for i in range(self.n_steps):
            dx = dt * p / self.m
            x = x + dx
            disp = torch.maximum(disp, (x - x0).norm(dim=1).max())
            s1, f1 = self.surrogate(x)
            # the surrogate's energy change along the path (trapezoid rule
            # on its forces): smooth where the BF16 energies are not, and
            # odd under reversal of the trajectory
            w_atom = -0.5 * ((f + f1) * dx).double().sum(1)
            work.index_add_(0, self.cfg, w_atom)
            f = f1.clone()
            if i + 1 < self.n_steps:
                p = p + dt * f
        p = p + 0.5 * dt * f
        k1 = self._kinetic(p)
        dhs = work + (k1 - k0)
        e1 = self.pot.evaluate(x, want_grad=False)[0]
        dh = (e1 - self.E) + (k1 - k0)
        logu = torch.log(torch.rand((2, self.B), generator=self.gen,
                                    device=x.device, dtype=torch.float64))
        st1 = da_stage1(logu[0], dhs, self.kT)
        st2 = da_stage2(logu[1], dh, dhs, self.kT)
        acc = st1 & st2
        self.x.copy_(torch.where(acc[self.cfg][:, None], x, self.x))
        self.E.copy_(torch.where(acc, e1, self.E))
        self.accepted += acc.to(torch.int64)
        self.stage1 += st1.to(torch.int64)
        self.max_disp.copy_(torch.maximum(self.max_disp, disp))
        self.sum_dhs_err += ((dh - dhs) ** 2).sum()
        self.sum_work_err += ((s1 - s0 - work) ** 2).sum()
        if self.buf_size:
            idx = (self.buf_ptr + torch.arange(self.B, device=x.device)
                   ) % self.buf_size
            self.buf_x[idx] = x.reshape(self.B, self.n_per, 3)
            self.buf_e[idx] = e1 / self.pot.conv
            self.buf_ptr.add_(self.B)

    def _capture(self):
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        state = (self.x.clone(), self.E.clone())
        rng = self.gen.get_state()
        with torch.cuda.stream(s):
            for _ in range(2):      # warm layouts, workspaces and buffers
                self._iteration()
        torch.cuda.current_stream().wait_stream(s)
        # the warm-up consumed no step of the chains
        self.x.copy_(state[0])
        self.E.copy_(state[1])
        self.gen.set_state(rng)
        self._reset_counters()
        self.graph = torch.cuda.CUDAGraph()
        if hasattr(self.graph, 'register_generator_state'):
            self.graph.register_generator_state(self.gen)
        with torch.cuda.graph(self.graph):
            self._iteration()

    def _reset_counters(self):
        self.accepted.zero_()
        self.stage1.zero_()
        self.max_disp.zero_()
        self.max_cnt.zero_()
        self.sum_dhs_err.zero_()
        self.sum_work_err.zero_()
        self.buf_ptr.zero_()
        self.proposed = 0
        self.buf_n = 0

    # ----------------------------------------------------------------- API
    def step(self, n=1):
        for _ in range(n):
            if self.graph is not None:
                self.graph.replay()
            else:
                self._iteration()
            self.proposed += 1
            self.buf_n = min(self.buf_n + self.B, self.buf_size)
        return self

    def check(self):
        """Raise if a neighbour list overflowed or an atom moved more than
        half the skin within a trajectory (the lists would have missed
        pairs)."""
        mc, md = int(self.max_cnt.item()), float(self.max_disp.item())
        if mc > self.max_nb:
            raise NativeError(f'neighbour list overflow: {mc} > {self.max_nb}')
        if md >= 0.5 * self.skin:
            raise NativeError(f'an atom moved {md:.3f} A within a trajectory '
                              f'(skin {self.skin} A)')
        return {'max_neighbours': mc, 'max_displacement': md}

    def train(self, steps=1, batch=32):
        """``steps`` Adam steps on one random batch of exact (configuration,
        Rw) pairs of the replay buffer (descriptors computed once for the
        batch); the iteration then uses the new weights."""
        if self.buf_n < 2:
            return None
        b = min(int(batch), self.buf_n)
        off = (np.arange(b + 1) * self.n_per).astype(np.int32)
        idx = torch.randint(0, self.buf_n, (b,), generator=self.gen,
                            device=self.x.device)
        fb = self.sur.features(self.buf_x[idx].reshape(-1, 3), off)
        target = self.buf_e[idx]
        loss = None
        for _ in range(int(steps)):
            loss = self.sur.train_step(fb, off, target)
        self.refresh_weights()
        return loss

    def acceptance(self):
        n = max(self.proposed, 1)
        return {'accepted': (self.accepted.double() / n).cpu().numpy(),
                'stage1': (self.stage1.double() / n).cpu().numpy()}

    def positions(self):
        return self.x
