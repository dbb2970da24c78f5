"""Recursive No-U-Turn sampler (TEST INFRASTRUCTURE: only tests/ use it).

Hoffman and Gelman, JMLR 15 (2014), Algorithm 3 (efficient NUTS: BuildTree
by recursion, the proposal of a doubled subtree kept with probability
n'/(n' + n'')), Algorithm 4 (first step size) and Algorithm 6 (dual
averaging), with the conventions of pyIID's NUTSCanonicalEnsemble
(pyiid/sim/nuts_hmc.py:15-232):

* total energies H = U + K compared without a temperature factor; slice
  u ~ U(0, 1): in the slice when u <= exp(H0 - H), growth stops when
  u >= exp(Emax + H0 - H), Emax = 200 (nuts_hmc.py:46-60);
* leaf statistic min(1, exp(H_before - H_leaf)) (nuts_hmc.py:61-63);
* U-turn test span . v >= 0 at both ends of a subtree, span = x_pos - x_neg
  (nuts_hmc.py:82-86, 206-210);
* Maxwell-Boltzmann momenta rescaled to exactly kT per degree of freedom,
  the escape depth, and dual averaging with mu = log(10 eps0), gamma =
  0.05, t0 = 10 on the last subtree's statistic (nuts_hmc.py:100-232);
* pyIID's leapfrog with re-centring and evaluation at the centred point
  (pyiid/sim/__init__.py:10-38).

It reads its random numbers from the same keyed per-iteration tables as the
product's iterative engine (pyiid_gb300.nuts): normals then a table of
uniforms per iteration, slots u, directions, acceptances and one merge per
internal tree node.  The recursion below is therefore an independent
formulation of the same sampler, against which the engine's leaf-by-leaf
tree growth is checked decision for decision.
"""
import numpy as np

KB = 1.380649e-23 / 1.602176634e-19  # eV / K (SI 2019 exact values)
EMAX = 200.0


def n_slots(J):
    return 1 + 2 * J + (2 ** J - 1 - J)


class RecursiveNUTS:
    """One chain.  potential(x [N, 3]) -> (U, F [N, 3])."""

    def __init__(self, potential, x0, masses, temperature, seed, J,
                 accept_target=0.65):
        self.pot = potential
        self.m = np.asarray(masses, np.float64)[:, None]
        self.kT = temperature * KB
        self.J = J
        self.delta = accept_target
        self.rs = np.random.RandomState(seed)
        self.x = np.asarray(x0, np.float64).copy()
        self.U, self.F = self.pot(self.x)
        self.samples, self.leapfrogs, self.accepted = [], 0, 0
        self.eps = self._first_step()
        self.leapfrogs = 0  # count the tree's steps only
        self.mu = np.log(10 * self.eps)
        self.hbar, self.m_it = 0.0, 0

    # ---------------------------------------------------------- pieces
    def K(self, p):
        return 0.5 * float((p * p / self.m).sum())

    def momenta(self, g):
        p = g * np.sqrt(self.m * self.kT)
        cur = 2 * self.K(p) / (3 * len(p))
        return p * np.sqrt(self.kT / cur) if cur > 0 else p

    def leapfrog(self, st, h):
        x, p, U, F = st
        p = p + 0.5 * h * F
        x = x + h * p / self.m
        U, F = self.pot(x)
        p = p + 0.5 * h * F
        x = x - 0.5 * (x.min(0) + x.max(0))
        U, F = self.pot(x)
        self.leapfrogs += 1
        return (x, p, U, F)

    def H(self, st):
        return st[2] + self.K(st[1])

    def no_uturn(self, neg, pos):
        span = (pos[0] - neg[0]).ravel()
        return (span.dot((neg[1] / self.m).ravel()) >= 0 and
                span.dot((pos[1] / self.m).ravel()) >= 0)

    def _first_step(self):
        p0 = self.momenta(self.rs.standard_normal(self.x.shape))
        st = (self.x, p0, self.U, self.F)
        H0 = self.H(st)

        def ratio(e):
            with np.errstate(over='ignore'):
                return np.exp(-self.H(self.leapfrog(st, e)) + H0)
        eps = 0.5
        r = ratio(eps)
        a = 1.0 if r > 0.5 else -1.0
        while r ** a > 2.0 ** -a:
            eps *= 2.0 ** a
            r = ratio(eps)
            if eps < 1e-7 or eps > 1e7:
                eps = 1.0
                break
        return eps

    # ---------------------------------------------------- Algorithm 3
    def build(self, st, v, j, depth, level_index):
        """Subtree of ``level`` j, node ``level_index`` inside the top
        subtree of depth ``depth``: returns (neg, pos, proposal, n, s,
        alpha_sum, n_alpha)."""
        if j == 0:
            leaf = self.leapfrog(st, v * self.eps)
            h = self.H(leaf)
            with np.errstate(over='ignore'):
                n = int(self.u <= np.exp(self.H0 - h))
                s = int(self.u < np.exp(EMAX + self.H0 - h))
                a = np.exp(-h + self.H(st))
            a = a if a < 1 else 1.0
            return leaf, leaf, leaf, n, s, a, 1
        neg, pos, prop, n1, s1, a1, na1 = self.build(st, v, j - 1, depth,
                                                     2 * level_index)
        if s1 == 1:
            edge = neg if v < 0 else pos
            neg2, pos2, prop2, n2, s2, a2, na2 = self.build(
                edge, v, j - 1, depth, 2 * level_index + 1)
            if v < 0:
                neg = neg2
            else:
                pos = pos2
            slot = (1 + 2 * self.J + (2 ** depth - 1 - depth)
                    + (2 ** (depth - j) - 1) + level_index)
            if self.tab[slot] < n2 / max(n1 + n2, 1):
                prop = prop2
            a1, na1 = a1 + a2, na1 + na2
            s1 = s2 * int(self.no_uturn(neg, pos))
            n1 = n1 + n2
        return neg, pos, prop, n1, s1, a1, na1

    # ---------------------------------------------------- Algorithm 6
    def iterate(self):
        g = self.rs.standard_normal(self.x.shape)
        self.tab = self.rs.random_sample(n_slots(self.J))
        p = self.momenta(g)
        st = (self.x, p, self.U, self.F)
        self.H0 = self.H(st)
        self.u = self.tab[0]
        neg = pos = st
        n, s, j = 1, 1, 0
        while s == 1:
            v = -1.0 if self.tab[1 + j] < 0.5 else 1.0
            edge = neg if v < 0 else pos
            nneg, npos, prop, n1, s1, a, na = self.build(edge, v, j, j, 0)
            if v < 0:
                neg = nneg
            else:
                pos = npos
            r = n1 / n
            if s1 == 1 and self.tab[1 + self.J + j] < (r if r < 1 else 1.0):
                self.x, self.U, self.F = prop[0], prop[2], prop[3]
                self.samples.append(self.x.copy())
                self.accepted += 1
            n += n1
            s = s1 * int(self.no_uturn(neg, pos))
            j += 1
            if j >= self.J:
                s = 0
        w = 1.0 / (self.m_it + 10.0)
        self.hbar = (1 - w) * self.hbar + w * (self.delta - a / na)
        self.eps = float(np.exp(self.mu - np.sqrt(self.m_it) / 0.05 *
                                self.hbar))
        self.m_it += 1
