"""No-U-Turn sampling of many chains at once, with the tree on the device.

The sampler is the efficient No-U-Turn sampler with dual-averaging step-size
adaptation of Hoffman and Gelman (JMLR 15, 2014; Algorithms 3, 4 and 6),
with the conventions pyIID uses for it (pyiid/sim/nuts_hmc.py:15-232):

* energies are the calculator's total energies H = U + K in eV, compared
  without a temperature factor; the temperature enters only through the
  Maxwell-Boltzmann momenta (rescaled to exactly kT per degree of freedom),
  drawn afresh at every iteration;
* the slice variable u ~ U(0, 1) is compared in post-exponential form:
  a leaf is in the slice when u <= exp(H0 - H), and the tree stops growing
  once u >= exp(Emax + H0 - H), Emax = 200;
* the per-leaf acceptance statistic is min(1, exp(H_before - H_leaf)), the
  energy change of that leaf's own leapfrog step;
* the dual-averaging target uses the statistic of the last subtree of an
  iteration; log step = mu - sqrt(m)/gamma * hbar with mu = log(10 eps0),
  gamma = 0.05, t0 = 10, m counted from 0, no final averaging;
* the trajectory doubles at most ``escape_level`` times per iteration;
* every proposal a doubling accepts becomes a sample (an iteration can
  produce several), and the next iteration starts from the last one;
* the leapfrog is pyIID's (pyiid/sim/__init__.py:10-38): half kick, drift,
  half kick with the forces there, then the particle is re-centred on the
  origin (each axis shifted by minus the midpoint of its extent);
* the first step size comes from the doubling/halving search of
  Algorithm 4 on the energy ratio exp(H - H') from eps = 0.5, with a step
  outside [1e-7, 1e7] replaced by 1.

Instead of recursion, a subtree of depth j is grown leaf by leaf.  The leaf
index in binary says which completed subtrees merge when a leaf lands: the
stack of completed first halves, one per level, is the recursion's call
stack.  A first half whose U-turn flag is off ends its subtree early (its
second half is never built) and is carried up unchanged; a second half
merges with the stored first half of its level (Algorithm 3: the proposal
moves to the second half with probability n''/(n' + n''), counts and
acceptance statistics add, and the merged subtree stops on a U-turn between
its first and last leaf).  So the state of every chain is a fixed set of
tensors, and one "tick" advances every chain by one leapfrog step: one
batched energy-and-force evaluation plus a fixed sequence of tensor
operations, with no per-leaf exchange with the host.  Chains of different
tree shapes, depths and iteration counts run in lock step under masks.
Proposals are referenced by index (the leaf of this tick or a stack level),
so a tree level costs a few [B]-sized operations; the U-turn products
against every stack level are formed once per tick.

Randomness is keyed, not sequential: at the start of iteration it, chain c
draws, from its own ``numpy.random.RandomState(seed_c)``, the N x 3 normals
of its momenta and then one table of uniforms whose slots are fixed: u, one
direction per depth, one top-level acceptance per depth, and one merge
decision per internal node of every depth's subtree.  Whatever order the
device evaluates the tree in, every decision reads its own slot, so a chain
of a batch and the same chain run alone make the same decisions.
"""
import numpy as np
import torch

from .atoms import kB

__all__ = ['NUTSEngine', 'BatchedNUTS', 'Emax', 'n_table_slots']

Emax = 200.0


# ------------------------------------------------------------ table slots
def n_table_slots(escape_level):
    """Uniforms per chain and iteration: u, J directions, J acceptances and
    one merge per internal node of the subtrees of depth 0 .. J-1."""
    J = int(escape_level)
    return 1 + 2 * J + (2 ** J - 1 - J)


def slot_direction(J, j):
    """Direction of the doubling at depth j (< 0.5: backwards)."""
    return 1 + j


def slot_accept(J, j):
    """Top-level acceptance of the subtree of depth j."""
    return 1 + J + j


def slot_merge(J, j, level, index):
    """Merge forming node ``index`` (0-based, in time order) of ``level``
    (1 .. j) inside the subtree of depth j: heap numbering within the
    subtree (root 0), after the nodes of all shallower subtrees."""
    return 1 + 2 * J + (2 ** j - 1 - j) + (2 ** (j - level) - 1) + index


def _min1(x):
    """min(1, x) as Python's min evaluates it (NaN gives 1)."""
    return torch.where(x < 1, x, torch.ones_like(x))


class NUTSEngine:
    """Batched NUTS state machine on torch tensors (CPU or GPU).

    evaluate : callable x [B, N, 3] -> (U [B], F [B, N, 3]) (F: the forces
               the leapfrog kicks with, as the calculator defines them)
    x0       : start positions [B, N, 3]
    masses   : [B, N] or [N] (amu)
    seeds    : B integers (one RandomState per chain)
    reevaluate_centred : evaluate again at the re-centred leapfrog end point
               (what a calculator does when the positions move; needed for
               potentials that are not translation invariant)
    momentum : None for Maxwell-Boltzmann momenta at ``temperature``, else
               unit normal momenta (the reference's ``momentum`` option)
    """

    def __init__(self, evaluate, x0, masses, temperature, seeds,
                 escape_level=13, accept_target=0.65, momentum=None,
                 reevaluate_centred=True, dtype=torch.float64, device=None,
                 find_step_size=True):
        if not torch.is_tensor(x0):
            x0 = torch.as_tensor(np.asarray(x0, np.float64))
        x0 = x0.to(dtype=dtype, device=device)
        if x0.dim() != 3 or x0.shape[2] != 3:
            raise ValueError(f'x0 must be [B, N, 3] (got {list(x0.shape)})')
        B, N = int(x0.shape[0]), int(x0.shape[1])
        self.B, self.N, self.dtype, self.device = B, N, dtype, x0.device
        dev = self.device
        m = torch.as_tensor(np.asarray(masses, np.float64), dtype=dtype,
                            device=dev)
        if m.dim() == 1:
            m = m[None].expand(B, N)
        self.masses = m.reshape(B, N, 1).contiguous()
        self._evaluate = evaluate
        self.kT = float(temperature) * kB
        self.J = J = int(escape_level)
        if J < 1 or J > 20:
            raise ValueError('escape_level must be in [1, 20]')
        self.n_slots = n_table_slots(J)
        self.accept_target = float(accept_target)
        self.momentum = momentum
        self.reevaluate = bool(reevaluate_centred)
        seeds = [int(s) for s in seeds]
        if len(seeds) != B:
            raise ValueError('one seed per chain')
        self.seeds = seeds
        self.rs = [np.random.RandomState(s) for s in seeds]
        self.gamma, self.t0 = 0.05, 10.0
        self.evaluations = 0
        self.ar = torch.arange(B, device=dev)
        f = dict(dtype=dtype, device=dev)
        i64 = dict(dtype=torch.int64, device=dev)
        # current sample (the state an iteration starts from)
        self.x = x0.clone()
        U, F = self.evaluate(self.x)
        self.U, self.F = U.clone(), F.clone()
        # per-chain counters
        self.hbar = torch.zeros(B, **f)
        self.m_it = torch.zeros(B, **i64)
        self.iteration = torch.zeros(B, **i64)
        self.accepted = torch.zeros(B, **i64)
        self.leapfrogs = torch.zeros(B, **i64)
        self.samples_total = torch.zeros(B, **i64)
        self.samples = [[] for _ in range(B)]
        self.sample_energies = [[] for _ in range(B)]
        # tree state: edges (neg, pos) and the front (the last leaf), each
        # x, p, F [B, N, 3] and U, H [B]
        z3 = lambda: torch.zeros((B, N, 3), **f)  # noqa: E731
        self.ex = {s: z3() for s in ('neg', 'pos', 'front')}
        self.ep = {s: z3() for s in ('neg', 'pos', 'front')}
        self.eF = {s: z3() for s in ('neg', 'pos', 'front')}
        self.eU = {s: torch.zeros(B, **f) for s in ('neg', 'pos', 'front')}
        self.eH = {s: torch.zeros(B, **f) for s in ('neg', 'pos', 'front')}
        # stack levels 0..J-1 and the leaf of the tick (index J)
        self.first_x = torch.zeros((J + 1, B, N, 3), **f)
        self.first_p = torch.zeros((J + 1, B, N, 3), **f)
        self.prop_x = torch.zeros((J + 1, B, N, 3), **f)
        self.prop_F = torch.zeros((J + 1, B, N, 3), **f)
        self.prop_U = torch.zeros((J + 1, B), **f)
        self.stk_n = torch.zeros((J, B), **f)
        self.stk_s = torch.zeros((J, B), dtype=torch.bool, device=dev)
        self.stk_asum = torch.zeros((J, B), **f)
        self.stk_na = torch.zeros((J, B), **f)
        # iteration scalars
        self.H0 = torch.zeros(B, **f)
        self.u = torch.zeros(B, **f)
        self.n_tot = torch.ones(B, **f)
        self.j = torch.zeros(B, **i64)
        self.leaf = torch.zeros(B, **i64)
        self.v = torch.ones(B, **f)
        self.tab = torch.zeros((B, self.n_slots), **f)
        if find_step_size:
            self.step = self.find_step_size().clone()
        else:
            self.step = torch.full((B,), 0.5, **f)
        self.mu = torch.log(10 * self.step)
        self._cap = 0

    # ------------------------------------------------------------ helpers
    def evaluate(self, x):
        self.evaluations += 1
        U, F = self._evaluate(x)
        return (U.to(self.dtype).reshape(self.B),
                F.to(self.dtype).reshape(self.B, self.N, 3))

    def kinetic(self, p):
        return 0.5 * (p * p / self.masses).flatten(1).sum(1)

    def _momenta(self, g):
        """Momenta [B, N, 3] from normals g: Maxwell-Boltzmann at kT,
        rescaled so that 2 K / (3 N) = kT exactly; or g itself."""
        if self.momentum is not None:
            return g.clone()
        p = g * torch.sqrt(self.masses * self.kT)
        cur = 2 * self.kinetic(p) / (3 * self.N)
        scale = torch.where(cur > 0, torch.sqrt(self.kT / cur),
                            torch.ones_like(cur))
        return p * scale[:, None, None]

    def _centre(self, x):
        return x - 0.5 * (x.amin(1, keepdim=True) + x.amax(1, keepdim=True))

    def leapfrog(self, x, p, F, h):
        """pyIID's leapfrog with signed step h [B]: (x', p', U', F')."""
        hh = h[:, None, None]
        p = p + 0.5 * hh * F
        x = x + hh * p / self.masses
        U, F = self.evaluate(x)
        p = p + 0.5 * hh * F
        x = self._centre(x)
        if self.reevaluate:
            U, F = self.evaluate(x)
        return x, p, U, F

    # ------------------------------------------------------ initial step
    def find_step_size(self):
        """Algorithm 4 with pyIID's energies (see the module docstring).
        The momenta are the first draw of each chain's random state."""
        g = torch.as_tensor(np.stack([r.standard_normal((self.N, 3))
                                      for r in self.rs]), dtype=self.dtype,
                            device=self.device)
        p0 = self._momenta(g)
        H0 = self.U + self.kinetic(p0)
        one = torch.ones(self.B, dtype=self.dtype, device=self.device)
        eps = 0.5 * one

        def ratio(e):
            _, p, U, _ = self.leapfrog(self.x, p0, self.F, e)
            return torch.exp(-(U + self.kinetic(p)) + H0)
        r = ratio(eps)
        a = torch.where(r > 0.5, one, -one)
        active = torch.ones(self.B, dtype=torch.bool, device=self.device)
        for _ in range(256):
            cont = active & (torch.pow(r, a) > torch.pow(2.0 * one, -a))
            if not bool(cont.any()):
                break
            eps = torch.where(cont, eps * torch.pow(2.0 * one, a), eps)
            r = torch.where(cont, ratio(eps), r)
            out = cont & ((eps < 1e-7) | (eps > 1e7))
            eps = torch.where(out, one, eps)
            active = cont & ~out
        return eps

    # ---------------------------------------------------------- iterations
    def _ensure_run_buffers(self, its):
        """Per-run random tables and the sample buffer, reused (and kept at
        fixed addresses for a captured tick) while they are large enough."""
        cap = getattr(self, '_cap', 0)
        if its <= cap:
            return
        B, dev, dt = self.B, self.device, self.dtype
        self._cap = its
        self._normals = torch.zeros((its, B, self.N, 3), dtype=dt, device=dev)
        self._tables = torch.zeros((its, B, self.n_slots), dtype=dt,
                                   device=dev)
        self._its = torch.zeros((), dtype=torch.int64, device=dev)
        self._base = torch.zeros(B, dtype=torch.int64, device=dev)
        self._target = torch.zeros(B, dtype=torch.int64, device=dev)
        S = its * self.J
        self._smp_x = torch.zeros((B, S, self.N, 3), dtype=dt, device=dev)
        self._smp_U = torch.zeros((B, S), dtype=dt, device=dev)
        self._smp_n = torch.zeros(B, dtype=torch.int64, device=dev)
        self._graph = None

    def run(self, iterations, graph=False):
        """Advance every chain by ``iterations`` iterations (chains that
        finish first idle under the mask).  With ``graph`` (CUDA only) one
        tick is captured once and replayed.  Returns the ticks taken."""
        B, its = self.B, int(iterations)
        if its < 1:
            return 0
        self._ensure_run_buffers(its)
        normals = np.empty((its, B, self.N, 3))
        tables = np.empty((its, B, self.n_slots))
        for c, rs in enumerate(self.rs):
            for t in range(its):
                normals[t, c] = rs.standard_normal((self.N, 3))
                tables[t, c] = rs.random_sample(self.n_slots)
        self._normals[:its].copy_(torch.as_tensor(normals, dtype=self.dtype))
        self._tables[:its].copy_(torch.as_tensor(tables, dtype=self.dtype))
        self._its.fill_(its)
        self._base.copy_(self.iteration)
        self._target.copy_(self.iteration + its)
        self._smp_n.zero_()
        self._start_iteration(torch.ones(B, dtype=torch.bool,
                                         device=self.device))
        use_graph = graph and self.device.type == 'cuda'
        if use_graph and self._graph is None:
            self._capture_tick()
        per_tick = 2 if self.reevaluate else 1
        ticks = 0
        while bool((self.iteration < self._target).any()):
            if use_graph:
                self._graph.replay()
                self.evaluations += per_tick
            else:
                self.tick()
            ticks += 1
        self._collect()
        return ticks

    def _capture_tick(self):
        """Capture one tick.  The warm-up tick runs on a side stream on a
        copy of the state, which is then restored, so capturing consumes no
        step of the chains."""
        saved = self._state_tensors()
        backup = [t.clone() for t in saved]
        ev = self.evaluations
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self.tick()
        torch.cuda.current_stream().wait_stream(s)
        for t, b in zip(saved, backup):
            t.copy_(b)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.tick()
        for t, b in zip(saved, backup):
            t.copy_(b)
        self.evaluations = ev
        self._graph = g

    def _state_tensors(self):
        out = [self.x, self.U, self.F, self.hbar, self.m_it, self.iteration,
               self.accepted, self.leapfrogs, self.samples_total,
               self.first_x, self.first_p, self.prop_x, self.prop_F,
               self.prop_U, self.stk_n, self.stk_s, self.stk_asum,
               self.stk_na, self.H0, self.u, self.n_tot, self.j, self.leaf,
               self.v, self.tab, self.step, self._smp_x, self._smp_U,
               self._smp_n]
        for d in (self.ex, self.ep, self.eF, self.eU, self.eH):
            out.extend(d.values())
        return out

    def _start_iteration(self, mask):
        """New momenta, slice variable and depth-0 tree for chains in mask."""
        k = torch.minimum(self.iteration - self._base, self._its - 1
                          ).clamp(min=0)
        tab = self._tables[k, self.ar]
        p = self._momenta(self._normals[k, self.ar])
        H = self.U + self.kinetic(p)
        m1, m3 = mask, mask[:, None, None]
        self.tab.copy_(torch.where(mask[:, None], tab, self.tab))
        self.H0.copy_(torch.where(m1, H, self.H0))
        self.u.copy_(torch.where(m1, tab[:, 0], self.u))
        self.n_tot.copy_(torch.where(m1, torch.ones_like(self.n_tot),
                                     self.n_tot))
        self.j.copy_(torch.where(m1, torch.zeros_like(self.j), self.j))
        self.leaf.copy_(torch.where(m1, torch.zeros_like(self.leaf),
                                    self.leaf))
        v0 = torch.where(tab[:, slot_direction(self.J, 0)] < 0.5, -1.0, 1.0
                         ).to(self.dtype)
        self.v.copy_(torch.where(m1, v0, self.v))
        for s in ('neg', 'pos', 'front'):
            self.ex[s].copy_(torch.where(m3, self.x, self.ex[s]))
            self.ep[s].copy_(torch.where(m3, p, self.ep[s]))
            self.eF[s].copy_(torch.where(m3, self.F, self.eF[s]))
            self.eU[s].copy_(torch.where(m1, self.U, self.eU[s]))
            self.eH[s].copy_(torch.where(m1, H, self.eH[s]))

    def tick(self):
        """One leapfrog step of every active chain and the tree updates."""
        B, J, dt, ar = self.B, self.J, self.dtype, self.ar
        act = self.iteration < self._target
        fx, fp, fF, fH = (self.ex['front'], self.ep['front'],
                          self.eF['front'], self.eH['front'])
        x1, p1, U1, F1 = self.leapfrog(fx, fp, fF, self.v * self.step)
        H1 = U1 + self.kinetic(p1)
        self.leapfrogs += act.to(torch.int64)
        dH = self.H0 - H1
        n_leaf = (self.u <= torch.exp(dH)).to(dt)
        s_leaf = self.u < torch.exp(Emax + dH)
        a_leaf = _min1(torch.exp(-H1 + fH))
        # the leaf is slot J of the proposal / first-leaf buffers
        self.first_x[J] = x1
        self.first_p[J] = p1
        self.prop_x[J] = x1
        self.prop_F[J] = F1
        self.prop_U[J] = U1
        # U-turn products of the last leaf against every level's first leaf:
        # a merged subtree spans first leaf -> last leaf in direction v
        vlast = (p1 / self.masses).flatten(1)
        span = (x1.flatten(1)[None] - self.first_x[:J].flatten(2))
        d_first = (span * (self.first_p[:J] / self.masses[None]).flatten(2)
                   ).sum(2)
        d_last = (span * vlast[None]).sum(2)
        vs = self.v[None]
        uturn_ok = ((vs * d_first) >= 0) & ((vs * d_last) >= 0)   # [J, B]
        # carry the leaf node up the levels
        n, s, asum, na = n_leaf, s_leaf, a_leaf, torch.ones_like(a_leaf)
        pidx = torch.full((B,), J, dtype=torch.int64, device=self.device)
        fidx = pidx.clone()
        climbing = act.clone()
        pos = self.leaf.clone()
        done = torch.zeros_like(act)
        store_lvl = torch.full_like(pidx, -1)
        for k in range(J + 1):
            top = climbing & (self.j == k)
            done = done | top
            climbing = climbing & ~top
            if k == J:
                break
            odd = (pos & 1) == 1
            # a completed first half waits on the stack for its second half;
            # one whose flag is off ends the subtree and goes up unchanged
            store = climbing & ~odd & s
            store_lvl = torch.where(store, torch.full_like(store_lvl, k),
                                    store_lvl)
            climbing = climbing & ~store
            merge = climbing & odd
            slot = (1 + 2 * J + (2 ** self.j - 1 - self.j) +
                    (2 ** (self.j - k - 1).clamp(min=0) - 1) + (pos >> 1))
            draw = self.tab[ar, slot.clamp(0, self.n_slots - 1)]
            tot = self.stk_n[k] + n
            take2 = draw < n / torch.clamp(tot, min=1.0)
            pidx = torch.where(merge & ~take2, torch.full_like(pidx, k), pidx)
            fidx = torch.where(merge, torch.full_like(fidx, k), fidx)
            s = torch.where(merge, s & uturn_ok[k], s)
            n = torch.where(merge, tot, n)
            asum = torch.where(merge, self.stk_asum[k] + asum, asum)
            na = torch.where(merge, self.stk_na[k] + na, na)
            pos = torch.where(climbing, pos >> 1, pos)
        # stores (after the loop: the node's proposal / first leaf may sit in
        # lower levels, which later leaves will overwrite)
        st = store_lvl >= 0
        lvl = store_lvl.clamp(min=0)
        m3 = st[:, None, None]
        for buf, idx in ((self.prop_x, pidx), (self.prop_F, pidx),
                         (self.first_x, fidx), (self.first_p, fidx)):
            src = buf[idx, ar]
            buf[lvl, ar] = torch.where(m3, src, buf[lvl, ar])
        self.prop_U[lvl, ar] = torch.where(st, self.prop_U[pidx, ar],
                                           self.prop_U[lvl, ar])
        self.stk_n[lvl, ar] = torch.where(st, n, self.stk_n[lvl, ar])
        self.stk_s[lvl, ar] = torch.where(st, s, self.stk_s[lvl, ar])
        self.stk_asum[lvl, ar] = torch.where(st, asum, self.stk_asum[lvl, ar])
        self.stk_na[lvl, ar] = torch.where(st, na, self.stk_na[lvl, ar])
        # the leaf is the new front of every active chain
        a1, a3 = act, act[:, None, None]
        self.ex['front'].copy_(torch.where(a3, x1, fx))
        self.ep['front'].copy_(torch.where(a3, p1, fp))
        self.eF['front'].copy_(torch.where(a3, F1, fF))
        self.eU['front'].copy_(torch.where(a1, U1, self.eU['front']))
        self.eH['front'].copy_(torch.where(a1, H1, fH))
        self.leaf.copy_(torch.where(act & ~done, self.leaf + 1, self.leaf))
        self._finish_subtree(done, n, s, asum, na, pidx)

    def _finish_subtree(self, done, n, s, asum, na, pidx):
        """Top level of Algorithm 6 for chains whose doubling just ended."""
        J, ar, dt = self.J, self.ar, self.dtype
        draw = self.tab[ar, (1 + J + self.j).clamp(max=self.n_slots - 1)]
        take = done & s & (draw < _min1(n / self.n_tot))
        px = self.prop_x[pidx, ar]
        pU = self.prop_U[pidx, ar]
        pF = self.prop_F[pidx, ar]
        self._record(take, px, pU)
        t3 = take[:, None, None]
        self.x.copy_(torch.where(t3, px, self.x))
        self.U.copy_(torch.where(take, pU, self.U))
        self.F.copy_(torch.where(t3, pF, self.F))
        self.accepted += take.to(torch.int64)
        self.n_tot.copy_(torch.where(done, self.n_tot + n, self.n_tot))
        # the doubling extended the tree on side v: that edge is the front
        for side, msk in (('neg', done & (self.v < 0)),
                          ('pos', done & (self.v > 0))):
            m3 = msk[:, None, None]
            self.ex[side].copy_(torch.where(m3, self.ex['front'],
                                            self.ex[side]))
            self.ep[side].copy_(torch.where(m3, self.ep['front'],
                                            self.ep[side]))
            self.eF[side].copy_(torch.where(m3, self.eF['front'],
                                            self.eF[side]))
            self.eU[side].copy_(torch.where(msk, self.eU['front'],
                                            self.eU[side]))
            self.eH[side].copy_(torch.where(msk, self.eH['front'],
                                            self.eH[side]))
        span = (self.ex['pos'] - self.ex['neg']).flatten(1)
        ok = (((span * (self.ep['neg'] / self.masses).flatten(1)).sum(1) >= 0) &
              ((span * (self.ep['pos'] / self.masses).flatten(1)).sum(1) >= 0))
        self.j.copy_(torch.where(done, self.j + 1, self.j))
        self.samples_total += torch.where(done, 2 ** self.j,
                                          torch.zeros_like(self.j))
        s_new = s & ok & (self.j < J)
        cont = done & s_new
        # next doubling: the direction of depth j, from that side's edge
        vj = torch.where(
            self.tab[ar, (1 + self.j).clamp(max=J)] < 0.5, -1.0, 1.0).to(dt)
        self.v.copy_(torch.where(cont, vj, self.v))
        self.leaf.copy_(torch.where(done, torch.zeros_like(self.leaf),
                                    self.leaf))
        back = (cont & (self.v < 0))
        fwd = (cont & (self.v > 0))
        for msk, side in ((back, 'neg'), (fwd, 'pos')):
            m3 = msk[:, None, None]
            self.ex['front'].copy_(torch.where(m3, self.ex[side],
                                               self.ex['front']))
            self.ep['front'].copy_(torch.where(m3, self.ep[side],
                                               self.ep['front']))
            self.eF['front'].copy_(torch.where(m3, self.eF[side],
                                               self.eF['front']))
            self.eU['front'].copy_(torch.where(msk, self.eU[side],
                                               self.eU['front']))
            self.eH['front'].copy_(torch.where(msk, self.eH[side],
                                               self.eH['front']))
        # iteration over: dual averaging on the last subtree's statistic
        over = done & ~s_new
        mf = self.m_it.to(dt)
        w = 1.0 / (mf + self.t0)
        hbar = (1 - w) * self.hbar + w * (self.accept_target - asum / na)
        step = torch.exp(self.mu - (torch.sqrt(mf) / self.gamma) * hbar)
        self.hbar.copy_(torch.where(over, hbar, self.hbar))
        self.step.copy_(torch.where(over, step, self.step))
        self.m_it += over.to(torch.int64)
        self.iteration += over.to(torch.int64)
        again = over & (self.iteration < self._target)
        self._start_iteration(again)

    def _record(self, take, px, pU):
        """Accepted proposals into the per-run sample buffer (device)."""
        ar = self.ar
        i = self._smp_n.clamp(max=self._smp_x.shape[1] - 1)
        t3 = take[:, None, None]
        self._smp_x[ar, i] = torch.where(t3, px, self._smp_x[ar, i])
        self._smp_U[ar, i] = torch.where(take, pU, self._smp_U[ar, i])
        self._smp_n += take.to(torch.int64)

    def _collect(self):
        """Move the run's samples into the per-chain lists."""
        counts = self._smp_n.cpu().tolist()
        if not any(counts):
            return
        xs = self._smp_x.cpu()
        us = self._smp_U.cpu()
        for c, k in enumerate(counts):
            for i in range(k):
                self.samples[c].append(xs[c, i].clone())
                self.sample_energies[c].append(float(us[c, i]))


class _ChainView:
    """Per-chain results of a :class:`BatchedNUTS`, named as the sequential
    sampler's attributes."""

    def __init__(self, engine, c):
        self._e, self._c = engine, c

    @property
    def samples(self):
        return [x.cpu().numpy() for x in self._e.samples[self._c]]

    @property
    def step_size(self):
        return float(self._e.step[self._c])

    @property
    def mu(self):
        return float(self._e.mu[self._c])

    @property
    def metadata(self):
        e, c = self._e, self._c
        return {'seed': e.seeds[c],
                'accepted_samples': int(e.accepted[c]),
                'samples_total': int(e.samples_total[c]),
                'leapfrog_steps': int(e.leapfrogs[c])}


class BatchedNUTS:
    """NUTS on the B configurations of one PDFPotential, all on the GPU.

    Energies are conv * potential and forces -1/2 conv dV/dx (Calc1D's
    convention, calc/calc_1d.py:89-95), so chain c reproduces a sequential
    :class:`pyiid_gb300.sim.nuts_hmc.NUTSCanonicalEnsemble` run with seed c
    on a Calc1D of the same potential.  ``exact`` re-evaluates the potential
    at the re-centred leapfrog end points as that calculator does (twice the
    evaluations); without it the drift point's values are kept (the Debye
    potential is translation invariant)."""

    def __init__(self, pot, starts, temperature=300.0, seeds=None,
                 escape_level=13, accept_target=0.65, exact=True,
                 graph=True):
        self.pot = pot
        self.graph = bool(graph)
        B = pot.n_configs
        starts = np.asarray(starts, np.float64).reshape(B, -1, 3)
        masses = np.asarray(pot.masses, np.float64).reshape(B, -1)
        out = pot.buffers()

        k = -0.5 * float(pot.conv)

        def evaluate(x):
            # as Calc1D: conv * Rw in FP64, forces (-1/2 conv) times the
            # float32 gradient of Rw, scaled in FP64
            e, _ = pot.evaluate(x.reshape(-1, 3).to(torch.float32), out=out)
            g = out['grad'].to(x.dtype)
            return e, (k * g).reshape(x.shape)

        seeds = list(range(B)) if seeds is None else list(seeds)
        self.engine = NUTSEngine(evaluate, torch.as_tensor(starts,
                                                           device=pot.device),
                                 masses, temperature, seeds,
                                 escape_level=escape_level,
                                 accept_target=accept_target,
                                 reevaluate_centred=exact,
                                 device=pot.device)
        self.chains = [_ChainView(self.engine, c) for c in range(B)]

    @property
    def evaluations(self):
        return self.engine.evaluations

    def step(self, iterations=1):
        return self.engine.run(iterations, graph=self.graph)

    def energies(self):
        return self.engine.U.cpu().numpy()

    def positions(self):
        return self.engine.x
