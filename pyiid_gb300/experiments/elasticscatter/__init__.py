"""Drop-in ``ElasticScatter`` whose processor is the GB300 library.

Mirrors pyiid/experiments/elasticscatter/__init__.py: the same constructor,
experiment dictionary, grids, per-atom scatter caching on the Atoms object,
getters and slicing.  The processor plug-in contract is the same three
callables (``self.fq``, ``self.grad``, ``self.grad_pdf``) plus the
``processor`` / ``alg`` tags (__init__.py:101-105, 206-292).

Processor selection: ``avail_pro = ['GB300']``.  The reference's 'MPI-GPU',
'Multi-GPU' and 'CPU' processors are not provided: ``set_processor`` returns
None for them, exactly as the reference does for a processor that is not
viable, and ``set_processor()`` raises if no GB300 is usable (there is no
CPU fallback).
"""
import math

import numpy as np

from .kernels.master_kernel import get_pdf_at_qmin
from ...scatter_factors import form_factor_array

__all__ = ['ElasticScatter', 'check_gpu', 'all_changes']

all_changes = ['positions', 'numbers', 'cell', 'pbc', 'charges', 'magmoms',
               'exp']


def check_gpu():
    """True when a GB300 (sm_103a) device and the library are usable."""
    try:
        from ..._native import context
        context()
        return True
    except Exception:  # noqa: BLE001
        return False


class ElasticScatter(object):
    """Theoretical powder diffraction / PDF of a set of atoms on one GB300.

    >>> from pyiid_gb300.atoms import Atoms
    >>> atoms = Atoms('Au4', [[0, 0, 0], [3, 0, 0], [0, 3, 0], [3, 3, 0]])
    >>> s = ElasticScatter({'rmax': 5., 'rmin': 2.})
    >>> gr = s.get_pdf(atoms)
    """

    def __init__(self, exp_dict=None, verbose=False, seed=None):
        self.verbose = verbose
        self.wrap_atoms_state = None
        if seed is None:
            self.seed = int(np.random.random() * 2 ** 32)
        elif isinstance(seed, int):
            self.seed = seed
        else:
            raise ValueError('Expected an integer!')
        self.rs = np.random.RandomState(self.seed)
        self.avail_pro = ['GB300']
        self.exp_dict_keys = ['qmin', 'qmax', 'qbin', 'rmin', 'rmax', 'rstep',
                              'sampling']
        self.default_values = [0.0, 25, .1, 0.0, 40.0, .01, 'full']
        self.alg = None
        self.processor = None
        self.exp = None
        self.pdf_qbin = None
        self.update_experiment(exp_dict)
        self.fq = None
        self.grad = None
        self.grad_pdf = None
        if self.set_processor() is None:
            raise RuntimeError(
                'no usable GB300 processor: pyiid_gb300 needs an sm_103a GPU '
                'and its native library (there is no CPU fallback)')

    # ------------------------------------------------------------ scatter
    def _wrap_atoms(self, atoms):
        """Per-atom scatter arrays as the reference builds them
        (__init__.py:110-151), plus the species column / per-species tables
        the GB300 processor consumes.

        Reproduced reference behaviours: both grids are evaluated at
        ``k * exp['qbin']`` (line 137), and element-table row i is evaluated
        for the i-th atom's number but assigned to ``list(set(numbers))[i]``
        (lines 123-143; only visible for multi-element systems whose first
        atoms are not one of each element in set order)."""
        if 'qbin' not in self.exp.keys():
            self.exp['qbin'] = .1
        n = len(atoms)
        e_num = atoms.get_atomic_numbers()
        e_list = list(set(e_num.tolist()))
        species = np.zeros(n, np.int32)
        for i, z in enumerate(e_list):
            species[np.where(atoms.numbers == z)[0]] = i
        tables = {}
        for qbin, name in zip([self.exp['qbin'], self.pdf_qbin],
                              ['F(Q) scatter', 'PDF scatter']):
            qmax_bin = int(math.floor(self.exp['qmax'] / qbin))
            q_eval = np.arange(qmax_bin) * self.exp['qbin']
            set_arr = np.zeros((len(e_list), qmax_bin), dtype=np.float32)
            for tx in range(len(e_list)):
                set_arr[tx] = form_factor_array(int(e_num[tx]), q_eval)
            scatter_array = np.zeros((n, qmax_bin), dtype=np.float32)
            for i in range(len(e_list)):
                scatter_array[np.where(atoms.numbers == e_list[i])[0], :] = \
                    set_arr[i, :]
            if name in atoms.arrays.keys():
                del atoms.arrays[name]
            atoms.set_array(name, scatter_array)
            tables[name] = set_arr if len(e_list) else np.zeros(
                (1, qmax_bin), np.float32)
        atoms.set_array('GB300 species', species)
        atoms.info['GB300 tables'] = tables
        atoms.info['exp'] = self.exp
        atoms.info['scatter_atoms'] = n

    def _check_wrap_atoms_state(self, atoms):
        """Refresh the atoms' scatter tables when they are stale; returns
        whether they were current (__init__.py:153-178)."""
        current = self.check_wrap_atoms_state(atoms)
        if not current:
            self._ensure(atoms, known_stale=True)
        return current

    def update_experiment(self, exp_dict):
        """__init__.py:180-204."""
        if exp_dict is None or bool(exp_dict) is False:
            exp_dict = {}
        for key, dv in zip(self.exp_dict_keys, self.default_values):
            if key not in exp_dict.keys():
                exp_dict[key] = dv
        if exp_dict['sampling'] == 'ns':
            exp_dict['rstep'] = np.pi / exp_dict['qmax']
        self.exp = exp_dict
        self.pdf_qbin = np.pi / (self.exp['rmax'] + 6 * 2 * np.pi /
                                 self.exp['qmax'])

    def set_processor(self, processor=None, kernel_type='flat'):
        """Select the processor (__init__.py:206-292).  Only 'GB300' exists;
        returns True on success and None for any other name."""
        if processor is None:
            for pro in self.avail_pro:
                if self.set_processor(processor=pro,
                                      kernel_type=kernel_type) is not None:
                    return True
            return None
        if processor == 'GB300' and check_gpu():
            from . import gb300_wrap
            self.fq = gb300_wrap.wrap_fq
            self.grad = gb300_wrap.wrap_fq_grad
            self.grad_pdf = gb300_wrap.grad_pdf
            self.processor = 'GB300'
            self.alg = 'flat'
            return True
        return None

    def check_wrap_atoms_state(self, atoms):
        """True when the atoms carry scatter tables made for this experiment
        and this number of atoms (__init__.py:294-302)."""
        info = atoms.info
        return bool(self.wrap_atoms_state is not None
                    and 'F(Q) scatter' in atoms.arrays
                    and info.get('exp') == self.exp
                    and info.get('scatter_atoms') == len(atoms))

    def _ensure(self, atoms, known_stale=False):
        if known_stale or not self.check_wrap_atoms_state(atoms):
            if self.verbose:
                print('calculating new scatter factors')
            self._wrap_atoms(atoms)
            self.wrap_atoms_state = atoms

    def _noisy(self, fq, iq_std, q, f_sq):
        """F(Q) plus Gaussian noise propagated from an I(Q) standard
        deviation: sigma_F = iq_std |Q| / |f^2| (__init__.py:332-341,
        :376-383), with a 1e-9 floor on a zero first point; one
        ``self.rs.normal`` draw of the whole vector."""
        sigma = iq_std * np.abs(q) / np.abs(f_sq)
        if sigma[0] == 0.0:
            sigma[0] = sigma[0] + 1e-9
        return fq + self.rs.normal(0, sigma)

    # ------------------------------------------------------------ getters
    def get_fq(self, atoms, iq_std=None, noise_distribution=None):
        """Reduced structure factor F(Q) (__init__.py:304-341): bins from
        qmin up; with ``iq_std`` the I(Q) noise carried through
        (avg f)^2."""
        self._ensure(atoms)
        k0 = int(np.floor(self.exp['qmin'] / self.exp['qbin']))
        fq = self.fq(atoms, self.exp['qbin'])[k0:]
        if iq_std is None:
            return fq
        f_avg = np.average(atoms.get_array('F(Q) scatter'), axis=0)
        return self._noisy(fq, iq_std, self.get_scatter_vector(),
                           (f_avg ** 2)[k0:])

    def get_pdf(self, atoms, iq_std=None, noise_distribution=np.random.normal):
        """Pair distribution function G(r) (__init__.py:343-391); with
        ``iq_std`` the I(Q) noise carried through avg(f^2) on the PDF grid.
        An ``iq_std`` array of another length is resampled linearly by
        index onto the grid's points (NaN beyond its last point); the
        reference's resampling line raises on current numpy."""
        self._ensure(atoms)
        fq = self.fq(atoms, self.pdf_qbin, 'PDF')
        if iq_std is not None:
            q = self.get_scatter_vector(pdf=True)
            f_sq = np.average(atoms.get_array('PDF scatter') ** 2, axis=0)
            if hasattr(iq_std, 'shape') and iq_std.shape != q.shape:
                src = np.asarray(iq_std, np.float64).ravel()
                at = np.arange(len(q), dtype=np.float64)
                iq_std = np.interp(at, np.arange(len(src)), src)
                iq_std[at > len(src) - 1] = np.nan
            fq = self._noisy(fq, iq_std, q, f_sq)
        return get_pdf_at_qmin(fq, self.exp['rstep'], self.pdf_qbin,
                               self.get_r(), self.exp['qmin'])

    def get_sq(self, atoms, iq_std=None, noise_distribution=np.random.normal):
        """Structure factor S(Q) (__init__.py:393-420)."""
        fq = self.get_fq(atoms, iq_std, noise_distribution)
        old_settings = np.seterr(all='ignore')
        sq = (fq / self.get_scatter_vector()) + np.ones(
            self.get_scatter_vector().shape)
        np.seterr(**old_settings)
        sq[np.isinf(sq)] = 0.
        return sq

    def get_iq(self, atoms, iq_std=None, noise_distribution=np.random.normal):
        """Scattering intensity I(Q) (__init__.py:422-446)."""
        sq = self.get_sq(atoms, iq_std, noise_distribution)
        f2 = np.average(atoms.get_array('F(Q) scatter'), axis=0) ** 2
        return sq * f2[int(np.floor(self.exp['qmin'] / self.exp['qbin'])):]

    def get_2d_scatter(self, atoms, pixel_array):
        """I(Q) projected onto a detector (__init__.py:448-475): a pixel of
        momentum transfer q takes the intensity of the bin Q_k with
        |q - Q_k| < qbin/2 (strictly; the higher bin where two qualify,
        0 where none does)."""
        iq = self.get_iq(atoms)
        qk = self.get_scatter_vector()
        nk = min(len(qk), len(iq))
        half = self.exp['qbin'] / 2.
        q = np.asarray(pixel_array, dtype=np.float64).ravel()
        img = np.zeros(q.shape)
        if nk == 0:
            return img.reshape(np.shape(pixel_array))
        with np.errstate(invalid='ignore'):
            near = np.floor((q - qk[0]) / self.exp['qbin'] + 0.5)
        near = np.nan_to_num(near, nan=-2.0, posinf=-2.0, neginf=-2.0)
        # the qualifying bins are among the nearest three; ascending order
        # lets the higher one win
        for dk in (-1, 0, 1):
            k = near.astype(np.int64) + dk
            kc = np.clip(k, 0, nk - 1)
            hit = ((k >= 0) & (k < nk) & (qk[kc] - half < q) &
                   (qk[kc] + half > q))
            img[hit] = iq[kc[hit]]
        return img.reshape(np.shape(pixel_array))

    def get_grad_fq(self, atoms):
        """Gradient of F(Q) in the reference convention (-1/2 dF/dx),
        [N, 3, K_ret] (__init__.py:477-496)."""
        self._ensure(atoms)
        g = self.grad(atoms, self.exp['qbin'])
        return g[:, :, int(np.floor(self.exp['qmin'] / self.exp['qbin'])):]

    def get_grad_pdf(self, atoms):
        """Gradient of G(r), [N, 3, R] (__init__.py:498-524)."""
        self._ensure(atoms)
        fq_grad = self.grad(atoms, self.pdf_qbin, 'PDF')
        qmin_bin = int(self.exp['qmin'] / self.pdf_qbin)
        fq_grad[:, :, :qmin_bin] = 0.
        rgrid = self.get_r()
        return self.grad_pdf(fq_grad, self.exp['rstep'], self.pdf_qbin, rgrid,
                             self.exp['qmin'])

    def get_scatter_vector(self, pdf=False):
        """Q grid (__init__.py:526-547)."""
        if pdf:
            return np.arange(0., math.floor(self.exp['qmax'] / self.pdf_qbin) *
                             self.pdf_qbin, self.pdf_qbin)
        return np.arange(self.exp['qmin'], math.floor(self.exp['qmax'] /
                                                      self.exp['qbin']) *
                         self.exp['qbin'], self.exp['qbin'])

    def get_r(self):
        """r grid (__init__.py:549-558)."""
        return np.arange(self.exp['rmin'], self.exp['rmax'], self.exp['rstep'])
