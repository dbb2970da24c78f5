"""Many NUTS chains advanced together on one GPU.

Each chain runs the reference's No-U-Turn sampler exactly
(pyiid/sim/nuts_hmc.py:15-232, as :mod:`pyiid_gb300.sim.nuts_hmc`
restates it): Maxwell-Boltzmann momenta, slice variable u in
post-exponential units, recursive tree doubling with the Emax = 200 slack,
the span U-turn criterion, the escape depth, the initial step-size search
and dual averaging.  The recursion of every chain is a Python generator that
yields at each leapfrog step; a scheduler gathers the pending leapfrog steps
of all chains and evaluates their end points as one batched exact
energy-and-gradient call (``pyiid_batch_potential_grad``), so the GPU sees
one launch sequence per tree leaf of the deepest chain instead of one per
leaf per chain.

Conventions are the reference's: energies conv * Rw (or chi^2), forces
-1/2 conv dV/dx (Calc1D's), ASE units, leapfrog with a centring step
(pyiid/sim/__init__.py:10-38), temperature entering through the momenta only.
Every chain owns a ``numpy.random.RandomState``, consumed in the reference's
order, so chain c of a batch reproduces a sequential
``NUTSCanonicalEnsemble`` run with the same seed and the same potential.
"""
import numpy as np
import torch

from .atoms import kB

__all__ = ['BatchedNUTS', 'Emax']

Emax = 200


class _State:
    """One point of phase space with its potential energy and forces."""
    __slots__ = ('x', 'p', 'U', 'F')

    def __init__(self, x, p, U, F):
        self.x, self.p, self.U, self.F = x, p, U, F


class _Chain:
    def __init__(self, masses, seed, temperature, escape_level,
                 accept_target, exact):
        self.exact = exact
        self.m = masses[:, None]
        self.rs = np.random.RandomState(seed)
        self.thermal_nrg = temperature * kB
        self.escape_level = escape_level
        self.accept_target = accept_target
        self.samples = []
        self.pe = []
        self.metadata = {'seed': seed, 'samples_total': 0,
                         'accepted_samples': 0}

    # ------------------------------------------------------- phase space
    def kinetic(self, p):
        return 0.5 * float((p * p / self.m).sum())

    def total(self, st):
        return st.U + self.kinetic(st.p)

    def velocities(self, st):
        return st.p / self.m

    def maxwell_boltzmann(self, n):
        """pyiid_gb300.atoms.MaxwellBoltzmannDistribution(force_temp=True)
        with this chain's random state."""
        temp = self.thermal_nrg
        p = self.rs.normal(size=(n, 3)) * np.sqrt(self.m * temp)
        if n:
            ke = self.kinetic(p)
            cur = 2 * ke / (3 * n)
            if cur > 0:
                p = p * np.sqrt(temp / cur)
        return p

    # ---------------------------------------------------- reference logic
    def leapfrog(self, st, step):
        """pyiid/sim/__init__.py:10-38: half kick, drift, half kick with the
        forces at the drifted positions, centring.  Yields the positions it
        needs evaluated and receives (U, F) there.  In exact mode the centred
        end point is evaluated again (the reference's calculator recomputes
        it there: the translation changes the float32 pair differences), else
        the drift point's values are kept for it."""
        p = st.p + 0.5 * step * st.F
        x = st.x + step * (p / self.m)
        U, F = yield x
        p = p + 0.5 * step * F
        x = x + (0.0 - 0.5 * (x.min(0) + x.max(0)))
        if self.exact:
            U, F = yield x
        return _State(x, p, U, F)

    def buildtree(self, st, u, v, j, e, e0):
        if j == 0:
            sp = yield from self.leapfrog(st, v * e)
            neg_delta_energy = e0 - self.total(sp)
            with np.errstate(over='ignore'):
                exp1 = np.exp(neg_delta_energy)
                exp2 = np.exp(Emax + neg_delta_energy)
            n_prime = int(u <= exp1)
            s_prime = int(u < exp2)
            with np.errstate(over='ignore'):
                a = min(1, np.exp(-self.total(sp) + self.total(st)))
            return sp, sp, sp, n_prime, s_prime, a, 1
        neg, pos, prop, n_p, s_p, a_p, na_p = yield from self.buildtree(
            st, u, v, j - 1, e, e0)
        if s_p == 1:
            if v == -1:
                neg, _, prop2, n_pp, s_pp, app, napp = \
                    yield from self.buildtree(neg, u, v, j - 1, e, e0)
            else:
                _, pos, prop2, n_pp, s_pp, app, napp = \
                    yield from self.buildtree(pos, u, v, j - 1, e, e0)
            if self.rs.uniform() < float(n_pp / (max(n_p + n_pp, 1))):
                prop = prop2
            a_p = a_p + app
            na_p = na_p + napp
            span = (pos.x - neg.x).flatten()
            s_p = s_pp * (span.dot(self.velocities(neg).flatten()) >= 0) * (
                span.dot(self.velocities(pos).flatten()) >= 0)
            n_p = n_p + n_pp
        return neg, pos, prop, n_p, s_p, a_p, na_p

    def find_step_size(self):
        """nuts_hmc.py:116-158 (with a Python +-1 exponent)."""
        st = _State(self.cur.x, self.maxwell_boltzmann(len(self.cur.x)),
                    self.cur.U, self.cur.F)
        step = .5
        sp = yield from self.leapfrog(st, step)
        with np.errstate(over='ignore'):
            a = 1.0 if np.exp(-self.total(sp) + self.total(st)) > 0.5 \
                else -1.0
            while np.exp(-self.total(sp) + self.total(st)) ** a > 2.0 ** -a:
                step *= 2 ** a
                sp = yield from self.leapfrog(st, step)
                if step < 1e-7 or step > 1e7:
                    step = 1.
                    break
        self.step_size = step
        self.mu = np.log(10 * step)
        self.sim_hbar = 0
        self.gamma = 0.05
        self.t0 = 10
        self.m_iter = 0

    def nuts_step(self):
        """nuts_hmc.py:160-232 for this chain."""
        cur = self.cur
        cur = _State(cur.x, self.maxwell_boltzmann(len(cur.x)), cur.U, cur.F)
        self.cur = cur
        u = self.rs.uniform(0, 1)
        e0 = self.total(cur)
        e = self.step_size
        n, s, j = 1, 1, 0
        neg = pos = cur
        a, na = 0.0, 1
        while s == 1:
            v = self.rs.choice([-1, 1])
            if v == -1:
                neg, _, prop, n_p, s_p, a, na = yield from self.buildtree(
                    neg, u, v, j, e, e0)
            else:
                _, pos, prop, n_p, s_p, a, na = yield from self.buildtree(
                    pos, u, v, j, e, e0)
            if s_p == 1 and self.rs.uniform() < min(1, n_p * 1. / n):
                self.cur = prop
                self.samples.append(prop.x.copy())
                self.pe.append(prop.U)
                self.metadata['accepted_samples'] += 1
            n = n + n_p
            span = (pos.x - neg.x).flatten()
            s = s_p * (span.dot(self.velocities(neg).flatten()) >= 0) * (
                span.dot(self.velocities(pos).flatten()) >= 0)
            j += 1
            self.metadata['samples_total'] += 2 ** j
            if j >= self.escape_level:
                s = 0
        w = 1. / (self.m_iter + self.t0)
        self.sim_hbar = (1 - w) * self.sim_hbar + w * (self.accept_target -
                                                       a / na)
        self.step_size = np.exp(self.mu - (self.m_iter ** .5 / self.gamma) *
                                self.sim_hbar)
        self.m_iter += 1


class BatchedNUTS:
    """NUTS chains over the configurations of a
    :class:`pyiid_gb300.sampling.PDFPotential` (all of the same atoms).

    positions : [B, N, 3]
    seeds     : B integers (one RandomState per chain)
    exact     : evaluate each leapfrog end point again after centring, as
                the reference does (two batched evaluations per tree leaf);
                False keeps the uncentred evaluation (one per leaf; equal up
                to float32 rounding of the translated pair differences)
    """

    def __init__(self, pot, positions, temperature=100, seeds=None,
                 escape_level=13, accept_target=.65, exact=True):
        self.pot = pot
        x = np.asarray(positions, np.float64)
        if x.ndim != 3 or x.shape[0] != pot.n_configs:
            raise ValueError('positions must be [n_configs, N, 3]')
        counts = np.diff(pot.offsets)
        if np.any(counts != x.shape[1]):
            raise ValueError('every configuration must have the same atoms')
        self.n_atoms = x.shape[1]
        if seeds is None:
            seeds = np.random.randint(0, 2 ** 31, pot.n_configs)
        masses = np.asarray(pot.masses[:self.n_atoms], np.float64)
        self.chains = [_Chain(masses, int(s), temperature, escape_level,
                              accept_target, exact) for s in seeds]
        self.evaluations = 0
        U, F = self._evaluate(x)
        for c, ch in enumerate(self.chains):
            ch.cur = _State(x[c].copy(), np.zeros_like(x[c]), U[c], F[c])
        self._run([ch.find_step_size() for ch in self.chains])

    def _evaluate(self, xs):
        """Energies conv * V and Calc1D forces -1/2 conv dV/dx of [B, N, 3]
        positions (one batched call; the same arithmetic as Calc1D's)."""
        from . import debye
        pot = self.pot
        pos = torch.as_tensor(np.asarray(xs, np.float32).reshape(-1, 3),
                              device=pot.device)
        out = debye.batch_potential_grad(
            pos, pot.species, pot.offsets, pot.table, pot.qstep,
            pot.exp['rstep'], pot.rgrid, pot.exp['qmin'], pot.gobs, pot.kind,
            out=pot.buffers())
        self.evaluations += 1
        U = out['energy'][:, 0].cpu().numpy() * pot.conv
        g = out['grad'].double().cpu().numpy().reshape(xs.shape)
        F = (-0.5 * pot.conv) * g
        return U, F

    def _run(self, gens):
        """Drive the chains' generators to completion, batching their
        leapfrog end points."""
        pending = {}
        for c, g in enumerate(gens):
            try:
                pending[c] = g.send(None)
            except StopIteration:
                pass
        xs = np.stack([ch.cur.x for ch in self.chains])
        while pending:
            for c, x in pending.items():
                xs[c] = x
            U, F = self._evaluate(xs)
            nxt = {}
            for c in pending:
                try:
                    nxt[c] = gens[c].send((U[c], F[c]))
                except StopIteration:
                    pass
            pending = nxt

    def step(self, n=1):
        """n NUTS iterations of every chain."""
        for _ in range(n):
            self._run([ch.nuts_step() for ch in self.chains])
        return self

    def positions(self):
        return np.stack([ch.cur.x for ch in self.chains])

    def energies(self):
        return np.array([ch.cur.U for ch in self.chains])

    def step_sizes(self):
        return np.array([ch.step_size for ch in self.chains])
