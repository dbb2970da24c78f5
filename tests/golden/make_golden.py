"""Generate golden vectors by running the reference pyIID code itself.

Run from the repository root:
    python tests/golden/make_golden.py REF_ROOT
or with PYIID_REFERENCE_ROOT=REF_ROOT in the environment, where REF_ROOT is the
root of a pyIID source checkout (the directory holding ``pyiid/``).
Writes tests/golden/reference_*.npz.

The reference is pure Python with numba-JIT'd loops.  numba, xraylib, mkl and
ASE are not installed, so this script registers small stand-in modules:
  * numba: ``jit`` / ``cuda.jit`` return the undecorated Python function (the
    reference's own CI runs exactly this way with NUMBA_DISABLE_JIT=1,
    .travis.yml), f4/i4 cast to numpy float32/int32, and ``cuda.gpus.lst``
    raises CudaSupportError so ElasticScatter selects its CPU processor;
  * xraylib.FF_Rayl: the stand-in form factor of pyiid_gb300.scatter_factors
    (form factors are an input of the path; the stand-in is used everywhere);
  * mkl: empty module;
and restores ``np.int`` (removed in numpy 2, used at
kernels/master_kernel.py:79).  The reference's ElasticScatter then runs its
default 'CPU'/'flat' processor (cpu_wrappers/flat_multi_cpu_wrap.py, a
multiprocessing Pool) and its master_kernel / calc functions unmodified.

Positions are given as float32 (the reference casts them anyway).
"""
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from pyiid_gb300.scatter_factors import form_factor  # noqa: E402


def install_stubs():
    class _NumType:
        def __init__(self, t):
            self.t = t

        def __call__(self, *a):
            return self.t(*a) if a else None

        def __getitem__(self, k):
            return self

    def jit(*args, **kwargs):
        if len(args) == 1 and callable(args[0]) and not kwargs and \
                not isinstance(args[0], _NumType):
            return args[0]
        return lambda f: f

    class CudaSupportError(Exception):
        pass

    class _Gpus:
        @property
        def lst(self):
            raise CudaSupportError('no CUDA in this stand-in')

    cuda = types.ModuleType('numba.cuda')
    cuda.jit = jit
    cuda.CudaSupportError = CudaSupportError
    cuda.gpus = _Gpus()
    numba = types.ModuleType('numba')
    numba.jit = jit
    numba.cuda = cuda
    for name, t in [('f4', np.float32), ('float32', np.float32),
                    ('f8', np.float64), ('float64', np.float64),
                    ('i4', np.int32), ('int32', np.int32),
                    ('i8', np.int64), ('int64', np.int64)]:
        setattr(numba, name, _NumType(t))
    numba.void = lambda *a, **k: None
    numba.__all__ = ['jit', 'cuda', 'f4', 'float32', 'f8', 'float64', 'i4',
                     'int32', 'i8', 'int64', 'void']
    sys.modules['numba'] = numba
    sys.modules['numba.cuda'] = cuda
    xraylib = types.ModuleType('xraylib')
    xraylib.FF_Rayl = lambda z, s: form_factor(int(z), float(s))
    sys.modules['xraylib'] = xraylib
    sys.modules['mkl'] = types.ModuleType('mkl')
    np.int = int


class MiniAtoms:
    """The parts of ase.Atoms that ElasticScatter touches."""

    def __init__(self, numbers, positions):
        self.numbers = np.asarray(numbers, dtype=np.int64)
        self.arrays = {'numbers': self.numbers,
                       'positions': np.asarray(positions, dtype=np.float64)}
        self.info = {}

    def __len__(self):
        return len(self.numbers)

    def get_positions(self):
        return self.arrays['positions'].copy()

    def get_atomic_numbers(self):
        return self.numbers.copy()

    def set_array(self, name, a):
        self.arrays[name] = a

    def get_array(self, name):
        return self.arrays[name].copy()


def case_positions():
    """Seeded positions (float32) for the golden cases."""
    rng = np.random.default_rng(20240601)
    sq = np.array([[0, 0, 0], [3, 0, 0], [0, 3, 0], [3, 3, 0]], np.float64)
    sq -= sq.mean(0)
    cases = {
        'au2': ([79, 79], np.array([[0, 0, 0], [3, 0, 0]], np.float32)),
        'square': ([79] * 4, sq.astype(np.float32)),
        'square75': ([79] * 4, (sq * .75).astype(np.float32)),
        'rand20': ([79] * 20, (rng.random((20, 3)) * 10).astype(np.float32)),
        'rand20b': ([79] * 20, (rng.random((20, 3)) * 10).astype(np.float32)),
        'alloy16': (list(rng.choice([78, 79], 16)),
                    (rng.random((16, 3)) * 8).astype(np.float32)),
        'rand40': ([79] * 40, (rng.random((40, 3)) * 12).astype(np.float32)),
    }
    base = cases['rand20'][1].astype(np.float64)
    cases['rand20p'] = ([79] * 20, (base + rng.normal(0, .05, base.shape))
                        .astype(np.float32))
    cases['alloy16p'] = (cases['alloy16'][0], (
        cases['alloy16'][1] + rng.normal(0, .05, (16, 3))).astype(np.float32))
    return cases


EXPS = {
    'default': None,
    # small r range so that [N, 3, R] gradients stay small
    'short': {'qmin': 0.6, 'qmax': 22.0, 'qbin': 0.13, 'rmin': 0.5,
              'rmax': 12.0, 'rstep': 0.05, 'sampling': 'full'},
    'ns': {'qmin': 1.1, 'qmax': 20.0, 'qbin': 0.1, 'rmin': 1.0,
           'rmax': 15.0, 'rstep': 0.02, 'sampling': 'ns'},
}


def main(ref_root):
    install_stubs()
    sys.path.insert(0, ref_root)
    from pyiid.experiments.elasticscatter import ElasticScatter
    from pyiid.calc import wrap_rw, wrap_grad_rw, wrap_chi_sq, \
        wrap_grad_chi_sq
    from pyiid.experiments.elasticscatter.kernels.master_kernel import \
        get_rw, get_chi_sq

    cases = case_positions()
    out = {}

    def run(tag, exp_name, numbers, pos, want_grad_pdf):
        scat = ElasticScatter(exp_dict=None if EXPS[exp_name] is None else
                              dict(EXPS[exp_name]))
        assert scat.processor == 'CPU' and scat.alg == 'flat'
        atoms = MiniAtoms(numbers, pos)
        key = f'{tag}__{exp_name}'
        out[key + '__numbers'] = np.asarray(numbers)
        out[key + '__positions'] = pos
        out[key + '__fq'] = scat.get_fq(atoms)
        out[key + '__sq'] = scat.get_sq(atoms)
        out[key + '__iq'] = scat.get_iq(atoms)
        out[key + '__pdf'] = scat.get_pdf(atoms)
        out[key + '__grad_fq'] = scat.get_grad_fq(atoms)
        out[key + '__fq_table'] = atoms.get_array('F(Q) scatter')
        out[key + '__pdf_table'] = atoms.get_array('PDF scatter')
        if want_grad_pdf:
            out[key + '__grad_pdf'] = scat.get_grad_pdf(atoms)
        out[key + '__r'] = scat.get_r()
        out[key + '__q'] = scat.get_scatter_vector()
        out[key + '__q_pdf'] = scat.get_scatter_vector(pdf=True)
        return scat, atoms

    for exp_name in ('default', 'short', 'ns'):
        for tag in ('au2', 'square', 'rand20', 'alloy16'):
            numbers, pos = cases[tag]
            run(tag, exp_name, numbers, pos,
                want_grad_pdf=(exp_name != 'default'))
    numbers, pos = cases['rand40']
    run('rand40', 'default', numbers, pos, False)

    # noisy getters (seeded RandomState of the ElasticScatter) and the
    # detector projection of I(Q)
    for exp_name in ('default', 'short'):
        numbers, pos = cases['alloy16']
        key = f'noise__alloy16__{exp_name}'
        e = EXPS[exp_name]
        scat = ElasticScatter(exp_dict=None if e is None else dict(e),
                              seed=1234)
        atoms = MiniAtoms(numbers, pos)
        out[key + '__fq_iq_std_scalar'] = scat.get_fq(atoms, iq_std=0.01)
        n_q = len(scat.get_scatter_vector())
        std = np.linspace(0.005, 0.02, n_q)
        out[key + '__iq_std_array'] = std
        out[key + '__fq_iq_std_array'] = scat.get_fq(atoms, iq_std=std)
        out[key + '__pdf_iq_std_scalar'] = scat.get_pdf(atoms, iq_std=0.01)
        n_qp = len(scat.get_scatter_vector(pdf=True))
        stdp = np.linspace(0.005, 0.02, n_qp)
        out[key + '__pdf_iq_std_array'] = scat.get_pdf(atoms, iq_std=stdp)
        prng = np.random.default_rng(77)
        q = scat.get_scatter_vector()
        pix = prng.uniform(q[0] - 1.0, q[-1] + 1.0, (40, 30))
        pix[0, :8] = q[:8]  # exactly on bin centres
        pix[1, :8] = q[:8] + scat.exp['qbin'] / 2.  # on bin edges
        out[key + '__pixels'] = pix
        out[key + '__2d'] = scat.get_2d_scatter(atoms, pix)

    # potentials through the calc wrappers (Calc1D's energy/forces path)
    for exp_name, (ta, tb) in [('short', ('square', 'square75')),
                               ('short', ('rand20', 'rand20b')),
                               ('ns', ('rand20', 'rand20b')),
                               ('short', ('rand20', 'rand20p')),
                               ('ns', ('rand20', 'rand20p')),
                               ('short', ('alloy16', 'alloy16p'))]:
        scat = ElasticScatter(exp_dict=dict(EXPS[exp_name]))
        na, pa = cases[ta]
        nb, pb = cases[tb]
        a1, a2 = MiniAtoms(na, pa), MiniAtoms(nb, pb)
        target = scat.get_pdf(a1)
        gcalc = scat.get_pdf(a2)
        gpdf = scat.get_grad_pdf(a2)
        key = f'pot__{ta}_{tb}__{exp_name}'
        out[key + '__target'] = target
        out[key + '__positions'] = pb
        out[key + '__numbers'] = np.asarray(nb)
        out[key + '__rw'] = np.array(wrap_rw(gcalc, target))
        # get_rw's optional per-point weights (no reference caller passes
        # them; the function accepts them): seeded weights in [0.2, 2)
        w = np.random.default_rng(17).uniform(0.2, 2.0, len(target))
        out[key + '__weight'] = w
        out[key + '__rw_weighted'] = np.array(get_rw(target, gcalc, weight=w))
        out[key + '__grad_rw'] = wrap_grad_rw(gpdf, gcalc, target)
        out[key + '__chi_sq'] = np.array(wrap_chi_sq(gcalc, target))
        out[key + '__grad_chi_sq'] = wrap_grad_chi_sq(gpdf, gcalc, target)

    # known-answer vectors of pyiid/tests/test_master/test_master_kernel.py
    x = np.arange(0, 2 * np.pi, .1)
    out['kat__rw_sin_cos'] = np.array(get_rw(np.sin(x), np.cos(x)))
    out['kat__rw_sin_sin'] = np.array(get_rw(np.sin(x), np.sin(x)))
    out['kat__chi_sin_cos'] = np.array(get_chi_sq(np.sin(x), np.cos(x)))
    out['kat__chi_sin_sin'] = np.array(get_chi_sq(np.sin(x), np.sin(x)))

    # the reference's carbon f(Q) table (one of its 60 identical rows)
    c60 = np.loadtxt(os.path.join(
        ref_root, 'pyiid/tests/test_master/c60_scat.txt'), dtype=np.float32)
    out['c60_row'] = c60[0]

    path = os.path.join(HERE, 'reference_vectors.npz')
    np.savez_compressed(path, **out)
    print('wrote', path, len(out), 'arrays',
          os.path.getsize(path) // 1024, 'KiB')


def reference_root(argv):
    """The pyIID checkout to run: the first argument, else
    $PYIID_REFERENCE_ROOT; fails with a message when neither names a
    directory holding the pyiid package."""
    root = argv[1] if len(argv) > 1 else os.environ.get('PYIID_REFERENCE_ROOT')
    if not root:
        sys.exit('usage: make_golden.py REF_ROOT (or set PYIID_REFERENCE_ROOT)'
                 ' -- the root of a pyIID source checkout')
    if not os.path.isdir(os.path.join(root, 'pyiid')):
        sys.exit(f'make_golden.py: {root!r} holds no pyiid/ package')
    return root


if __name__ == '__main__':
    main(reference_root(sys.argv))
