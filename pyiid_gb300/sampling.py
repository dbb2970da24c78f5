"""Device-resident PDF potential, its autograd wrapper, and batched HMC.

* :class:`PDFPotential` -- exact Rw (or chi^2) of many configurations against
  one observed G(r), with the exact position gradient from the hand-written
  adjoint kernel (one ``pyiid_batch_potential_grad`` call per evaluation).
* :func:`potential_energy` -- the same behind ``torch.autograd.Function``:
  forward returns the energies, backward is the adjoint gradient (no
  autograd graph through the kernels).
* :class:`BatchedHMC` -- many Hamiltonian Monte Carlo chains advanced in
  lock step on the GPU: Maxwell-Boltzmann momenta, velocity-Verlet
  trajectories (the leapfrog of pyiid/sim/__init__.py:10-38 and
  pyiid/sim/hmc.py:33-63), Metropolis accept/reject at temperature T.  With
  ``graph=True`` one whole iteration (momenta, trajectory, accept) is
  captured once in a CUDA graph and replayed.
* :class:`SingleAtomMC` -- single-atom Metropolis chains whose exact energy
  change costs O(N K) per proposal (``pyiid_mh_steps``): the raw Debye sums
  and the Gram form of the potential of every chain stay on the device and
  only the moved atom's pair terms are recomputed.

Units are ASE's: Angstrom, eV, amu; time unit Angstrom * sqrt(amu / eV).
The form factors of this API are species-correct (f evaluated at the PDF
grid's own Q values); the drop-in ElasticScatter keeps the reference's
table conventions instead.
"""
import math

import numpy as np
import torch

from . import debye
from .atoms import kB
from .scatter_factors import atomic_mass, form_factor_array

__all__ = ['PDFPotential', 'potential_energy', 'BatchedHMC',
           'SingleAtomMC', 'experiment_grids']


def experiment_grids(exp_dict=None):
    """(exp, pdf_qbin, n_bins, r grid) as ElasticScatter.update_experiment
    defines them (pyiid/experiments/elasticscatter/__init__.py:180-204)."""
    defaults = {'qmin': 0.0, 'qmax': 25, 'qbin': .1, 'rmin': 0.0,
                'rmax': 40.0, 'rstep': .01, 'sampling': 'full'}
    exp = dict(defaults)
    exp.update(exp_dict or {})
    if exp['sampling'] == 'ns':
        exp['rstep'] = np.pi / exp['qmax']
    qb = np.pi / (exp['rmax'] + 6 * 2 * np.pi / exp['qmax'])
    n_bins = int(math.floor(exp['qmax'] / qb))
    r = np.arange(exp['rmin'], exp['rmax'], exp['rstep'])
    return exp, qb, n_bins, r


class PDFPotential:
    """Exact PDF potential for B configurations of the same atom list.

    numbers : atomic numbers [N] (one configuration) -- every configuration
              has the same atoms; or a list of per-configuration arrays
              (uneven sizes allowed).
    gobs    : observed G(r) on the experiment's r grid.
    table   : optional form factors [number of distinct elements][n_bins]
              on the PDF grid (default: the stand-in f(Q) at the grid's Q).
    """

    def __init__(self, numbers, gobs, exp_dict=None, potential='rw',
                 conv=1.0, n_configs=1, device=None, table=None):
        self.exp, self.qstep, self.n_bins, self.rgrid = experiment_grids(
            exp_dict)
        if isinstance(numbers, (list, tuple)) and len(numbers) and \
                np.ndim(numbers[0]) == 1:
            per_cfg = [np.asarray(n) for n in numbers]
        else:
            per_cfg = [np.asarray(numbers)] * int(n_configs)
        allnum = np.concatenate(per_cfg) if per_cfg else np.zeros(0, int)
        self.uniq, sp = np.unique(allnum, return_inverse=True)
        self.species = sp.reshape(-1).astype(np.int32)
        self.offsets = np.concatenate(
            [[0], np.cumsum([len(n) for n in per_cfg])]).astype(np.int32)
        q = np.arange(self.n_bins) * self.qstep
        if table is not None:
            # explicit rows [len(unique numbers)][n_bins], e.g. the tables a
            # GB300 ElasticScatter attached to the atoms
            self.table = np.ascontiguousarray(table, np.float32)
            if self.table.shape != (max(len(self.uniq), 1), self.n_bins):
                raise ValueError(f'table shape {self.table.shape}, expected '
                                 f'({len(self.uniq)}, {self.n_bins})')
        else:
            self.table = np.stack([form_factor_array(z, q) for z in self.uniq]
                                  ).astype(np.float32) if len(self.uniq) else \
                np.zeros((1, self.n_bins), np.float32)
        self.masses = np.array([atomic_mass(z) for z in allnum])
        self.device = torch.device('cuda' if device is None else device)
        self.gobs = torch.as_tensor(np.asarray(gobs, np.float64),
                                    device=self.device)
        if self.gobs.shape[0] != len(self.rgrid):
            raise ValueError(f'gobs has {self.gobs.shape[0]} points, the r grid '
                             f'{len(self.rgrid)}')
        self.kind = potential
        self.conv = float(conv)
        self.n_configs = len(per_cfg)
        self.n_total = int(self.offsets[-1])
        self._out = None

    def config_index(self):
        """Configuration id of every packed atom (int64 CUDA tensor)."""
        counts = np.diff(self.offsets)
        return torch.as_tensor(np.repeat(np.arange(self.n_configs), counts),
                               device=self.device)

    def buffers(self):
        """Preallocated outputs (reused by every call; graph-safe)."""
        if self._out is None:
            d = self.device
            self._out = {
                'energy': torch.empty((self.n_configs, 2), dtype=torch.float64,
                                      device=d),
                'grad': torch.empty((self.n_total, 3), dtype=torch.float32,
                                    device=d),
                'gcalc': torch.empty((self.n_configs, len(self.rgrid)),
                                     dtype=torch.float64, device=d),
                'fq': torch.empty((self.n_configs, self.n_bins),
                                  dtype=torch.float32, device=d),
            }
        return self._out

    def evaluate(self, positions, want_grad=True, out=None):
        """Energies [B] (conv * potential, float64) and gradients dE/dx
        [sum N, 3] (float32, true gradient) of packed positions."""
        pos = positions.reshape(-1, 3)
        o = self.buffers() if out is None else out
        if not want_grad:
            o = dict(o)
            o['grad'] = None
        debye.batch_potential_grad(pos, self.species, self.offsets,
                                   self.table, self.qstep, self.exp['rstep'],
                                   self.rgrid, self.exp['qmin'], self.gobs,
                                   self.kind, want_grad=want_grad, out=o)
        e = o['energy'][:, 0] * self.conv
        g = o['grad'] * self.conv if want_grad else None
        return e, g


class _PotentialFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, positions, pot):
        e, g = pot.evaluate(positions.detach(), want_grad=True)
        ctx.save_for_backward(g.clone())
        ctx.cfg = pot.config_index()
        ctx.shape = positions.shape
        return e.clone()

    @staticmethod
    def backward(ctx, grad_e):
        (g,) = ctx.saved_tensors
        w = grad_e.to(g.dtype)[ctx.cfg][:, None]
        return (g * w).reshape(ctx.shape), None


def potential_energy(positions, pot):
    """Differentiable energies [B] of packed positions (gradient by the
    adjoint kernel)."""
    return _PotentialFn.apply(positions, pot)


class BatchedHMC:
    """Lock-step HMC chains over the configurations of a PDFPotential.

    dt        : leapfrog step (ASE time units)
    n_steps   : leapfrog steps per trajectory
    temperature : K; momenta ~ Maxwell-Boltzmann(T), acceptance
              min(1, exp(-(H1 - H0) / kB T))
    """

    def __init__(self, pot, positions, temperature=300.0, dt=1e-3,
                 n_steps=10, seed=0, graph=False):
        self.pot = pot
        d = pot.device
        self.kT = kB * float(temperature)
        self.dt = float(dt)
        self.n_steps = int(n_steps)
        self.x = torch.as_tensor(np.asarray(positions, np.float32),
                                 device=d).reshape(-1, 3).clone()
        m = torch.as_tensor(pot.masses, dtype=torch.float32, device=d)
        self.m = m[:, None]
        self.cfg = pot.config_index()
        self.gen = torch.Generator(device=d)
        self.gen.manual_seed(int(seed))
        self.accepted = torch.zeros(pot.n_configs, dtype=torch.int64, device=d)
        self.proposed = 0
        self.graph = None
        e, g = pot.evaluate(self.x)
        self.u = e.clone()
        self.g = g.clone()
        if graph:
            self._capture()

    def _kinetic(self, p):
        ke_atom = 0.5 * (p.double() ** 2 / self.m.double()).sum(1)
        out = torch.zeros(self.pot.n_configs, dtype=torch.float64,
                          device=p.device)
        return out.index_add_(0, self.cfg, ke_atom)

    def _iteration(self):
        p = torch.randn(self.x.shape, generator=self.gen,
                        device=self.x.device) * torch.sqrt(self.m * self.kT)
        h0 = self.u + self._kinetic(p)
        x = self.x.clone()
        g = self.g
        dt = self.dt
        p = p - 0.5 * dt * g
        for i in range(self.n_steps):
            x = x + dt * p / self.m
            e, g = self.pot.evaluate(x)
            if i + 1 < self.n_steps:
                p = p - dt * g
        p = p - 0.5 * dt * g
        h1 = e + self._kinetic(p)
        logu = torch.log(torch.rand(self.pot.n_configs, generator=self.gen,
                                    device=x.device, dtype=torch.float64))
        acc = logu < -(h1 - h0) / self.kT
        acc_atom = acc[self.cfg][:, None]
        self.x.copy_(torch.where(acc_atom, x, self.x))
        self.g.copy_(torch.where(acc_atom, g, self.g))
        self.u.copy_(torch.where(acc, e, self.u))
        self.accepted += acc.to(torch.int64)

    def _capture(self):
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            for _ in range(2):      # warm caches, layouts and buffers
                self._iteration()
        torch.cuda.current_stream().wait_stream(s)
        self.accepted.zero_()
        self.graph = torch.cuda.CUDAGraph()
        if hasattr(self.graph, 'register_generator_state'):
            self.graph.register_generator_state(self.gen)
        with torch.cuda.graph(self.graph):
            self._iteration()

    def step(self, n=1):
        for _ in range(n):
            if self.graph is not None:
                self.graph.replay()
            else:
                self._iteration()
            self.proposed += 1
        return self

    def acceptance(self):
        return (self.accepted.double() / max(self.proposed, 1)).cpu().numpy()

    def positions(self):
        return self.x.reshape(-1, 3)


class SingleAtomMC:
    """Single-atom Metropolis chains over the configurations of a
    PDFPotential, all on the device.

    Every step proposes, in every chain, one uniformly chosen atom and a
    displacement N(0, sigma^2) per coordinate, and accepts with probability
    min(1, exp(-(E' - E) / kT)), E = conv * potential -- the acceptance rule
    of the reference's Monte Carlo moves (pyiid/sim/hmc.py:66-92,
    pyiid/sim/gcmc.py:13-114) with the exact energy difference, obtained in
    O(N K) from the moved atom's pair terms instead of a full re-evaluation.

    graph : capture ``steps_per_replay`` steps once in a CUDA graph and
            replay it (the proposals depend only on (seed, chain, step), so
            graph and eager runs give identical chains).
    resync_every : steps between full exact re-evaluations of the running
            sums (bounds their FP64 drift; None disables).
    """

    def __init__(self, pot, positions, temperature=300.0, sigma=0.1, seed=0,
                 graph=False, steps_per_replay=32, resync_every=4096):
        self.pot = pot
        d = pot.device
        self.kT = kB * float(temperature)
        self.sigma = float(sigma)
        self.seed = int(seed)
        self.x = torch.as_tensor(np.asarray(positions, np.float32),
                                 device=d).reshape(-1, 3).clone()
        if self.x.shape[0] != pot.n_total:
            raise ValueError(f'{self.x.shape[0]} positions for '
                             f'{pot.n_total} atoms')
        self.state = {}
        self.resync_every = resync_every
        self.steps_per_replay = int(steps_per_replay)
        self.steps_done = 0
        self._since_sync = 0
        self.resync()
        self.state['counter'] = torch.zeros(pot.n_configs, dtype=torch.int64,
                                            device=d)
        self.state['accepted'] = torch.zeros(pot.n_configs,
                                             dtype=torch.int64, device=d)
        self._enqueue(0)  # sizes the context's buffers
        self.graph = None
        if graph:
            self._capture()

    def _enqueue(self, n, trace=None):
        p = self.pot
        debye.mh_steps(self.x, p.species, p.offsets, p.table, p.qstep,
                       p.exp['rstep'], p.rgrid, p.exp['qmin'], self.state, n,
                       p.conv, self.kT, self.sigma, self.seed, kind=p.kind,
                       trace=trace)

    def _capture(self):
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self._enqueue(self.steps_per_replay)

    def resync(self):
        """Recompute the running sums and energies of the current positions
        by a full exact evaluation."""
        p = self.pot
        debye.mh_init(self.x, p.species, p.offsets, p.table, p.qstep,
                      p.exp['rstep'], p.rgrid, p.exp['qmin'], p.gobs,
                      kind=p.kind, state=self.state)
        self._since_sync = 0

    def step(self, n=1, trace=None):
        """Advance every chain by n proposals.  ``trace`` (float64 CUDA
        tensor [n, B, 8]) records each proposal; it disables the graph."""
        done = 0
        while done < n:
            if self.resync_every and self._since_sync >= self.resync_every:
                self.resync()
            m = n - done
            if self.resync_every:
                m = min(m, self.resync_every - self._since_sync)
            if (self.graph is not None and trace is None and
                    m >= self.steps_per_replay):
                self.graph.replay()
                m = self.steps_per_replay
            else:
                tr = None if trace is None else trace[done:done + m]
                self._enqueue(m, tr)
            done += m
            self._since_sync += m
        self.steps_done += n
        return self

    def energies(self):
        """conv * potential of the current state of every chain [B]."""
        return self.state['energy'][:, 0] * self.pot.conv

    def acceptance(self):
        return (self.state['accepted'].double() /
                max(self.steps_done, 1)).cpu().numpy()

    def positions(self):
        return self.x

    def sums(self):
        """Running raw Debye sums S [B, K] (FP64, PDF grid)."""
        return debye.mh_views(self.state)['S']
