"""The C oracle (oracle/debye_ref.c) on the CPU: its FP64 sampled functions
against the NumPy oracle, and its FP32 port of the reference's default CPU
path (the timed CPU baseline) against the reference's own recorded
outputs."""
import numpy as np
import pytest

from oracle import debye_c as C
from oracle import debye_np as O
from pyiid_gb300 import structures as S
from pyiid_gb300.scatter_factors import species_tables

EXPS = {
    'default': None,
    'short': {'qmin': 0.6, 'qmax': 22.0, 'qbin': 0.13, 'rmin': 0.5,
              'rmax': 12.0, 'rstep': 0.05, 'sampling': 'full'},
    'ns': {'qmin': 1.1, 'qmax': 20.0, 'qbin': 0.1, 'rmin': 1.0,
           'rmax': 15.0, 'rstep': 0.02, 'sampling': 'ns'},
}


def rel(a, b):
    a = np.nan_to_num(np.asarray(a, np.float64))
    b = np.nan_to_num(np.asarray(b, np.float64))
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_sampled_sums_and_rows_match_the_numpy_oracle():
    """oracle_pair_sums / oracle_grad_rows (used for the sampled checks of
    large particles) equal the NumPy FP64 restatement on a 60-atom alloy."""
    pos = S.random_cube(60, 12.0, 4)
    nums = list(np.random.default_rng(3).choice([78, 79], 60))
    sp, tab, _ = species_tables(nums, 0.05, 300)
    bins = np.array([0, 1, 7, 150, 299], np.int32)
    s_c = C.pair_sums(pos, sp, tab, 0.05, bins)
    s_n = O.pair_sums(pos, tab[sp], 0.05)[bins]
    assert np.abs(s_c - s_n).max() <= 1e-12 * np.abs(s_n).max()
    atoms = np.array([0, 17, 59], np.int32)
    g_c = C.grad_rows(pos, sp, tab, 0.05, atoms)
    # the NumPy oracle returns -dS/dx / na, the reference's convention
    g_n = -O.grad_fq(pos, tab[sp], 0.05)[atoms] * O.normalization(tab[sp])
    assert rel(g_c[..., 1:], g_n[..., 1:]) <= 1e-12


def _port_grad(pos, per_atom, qbin):
    """wrap_fq_grad of the 'CPU' flat processor through the port:
    sum of the task gradients / na, nan_to_num
    (cpu_wrappers/flat_multi_cpu_wrap.py:63-102)."""
    n = len(pos)
    _, g, _ = C.port_tasks(pos, per_atom, qbin, 4096, n * (n - 1) // 2,
                           False, True)
    scat = np.asarray(per_atom, np.float32)
    i, j = np.tril_indices(n, -1)
    na = np.mean(scat[i] * scat[j], axis=0, dtype=np.float32) * np.float32(n)
    with np.errstate(all='ignore'):
        return np.nan_to_num(g / na)


def _scatter_keys(g):
    return sorted({k.rsplit('__', 1)[0] for k in g.files
                   if k.count('__') == 2 and not k.startswith(('pot', 'kat'))})


def test_fp32_port_matches_reference_outputs(golden):
    """The port's F(Q) and gradient equal the reference's recorded outputs
    to float32 rounding (observed <= 3e-8 norm-wise) for every scatter case
    of the golden file."""
    keys = _scatter_keys(golden)
    assert len(keys) == 13
    for key in keys:
        exp = O.update_experiment(EXPS[key.split('__')[1]])
        pos = golden[key + '__positions']
        ft = golden[key + '__fq_table']
        kq = int(np.floor(exp['qmin'] / exp['qbin']))
        f = C.port_fq(pos, ft, exp['qbin'])[kq:]
        assert rel(f, golden[key + '__fq']) <= 1e-7, key
        g = _port_grad(pos, ft, exp['qbin'])[:, :, kq:]
        assert rel(g, golden[key + '__grad_fq']) <= 1e-7, key


@pytest.mark.parametrize('chunk', [1, 7, 4096])
def test_port_task_split_does_not_change_the_sums(chunk):
    """The port's task split (one OpenMP thread per task) gives the same
    FP64 sums whatever the task size, to FP64 rounding of FP32 terms."""
    pos = S.random_cube(30, 10.0, 9)
    sp, tab, _ = species_tables([79] * 30, 0.1, 250)
    per_atom = tab[sp]
    s_ref, _, _ = C.port_tasks(pos, per_atom, 0.1, 435, 435, True, False)
    s, _, _ = C.port_tasks(pos, per_atom, 0.1, chunk, 435, True, False)
    assert np.abs(s - s_ref).max() <= 1e-12 * np.abs(s_ref).max()


@pytest.mark.parametrize('exp_name', ['default', 'short'])
def test_fp64_chain_compositions_match_the_numpy_oracle(exp_name):
    """The compositions the large-size GPU tests use (C pair sums -> F ->
    G -> potential, gradient rows through the adjoint vector, one moved
    atom's sum change) equal the NumPy oracle's full chain on a 50-atom
    alloy."""
    from oracle import mh_np
    exp = O.update_experiment(EXPS[exp_name])
    qb = O.pdf_qbin(exp)
    nb = int(np.floor(exp['qmax'] / qb))
    ref = S.fcc_nearest(4.08, 50)
    pos = S.displaced(ref, 0.05, 9)
    nums = list(np.random.default_rng(9).choice([78, 79], 50))
    sp, tab, _ = species_tables(nums, qb, nb)
    rg = O.r_grid(exp)
    gobs = O.pdf_tmatrix(O.fq(ref, tab[sp], qb), exp['rstep'], qb, rg,
                         exp['qmin'])
    f = C.fq_all_bins(pos, sp, tab, qb)
    assert rel(f, O.fq(pos, tab[sp], qb)) < 1e-12
    for kind in ('rw', 'chi_sq'):
        val, scale, gcalc, _, _ = C.potential_chain(pos, sp, tab, exp, qb,
                                                    gobs, kind)
        assert abs(val - O.potential_value(pos, tab[sp], exp, gobs, kind)) \
            <= 1e-12 * abs(val)
        atoms = np.array([0, 13, 49], np.int32)
        rows = C.true_grad_rows(pos, sp, tab, exp, qb, gobs, atoms, kind)
        _, tg = O.true_grad_potential(pos, tab[sp], exp, gobs, kind)
        assert rel(rows, tg[atoms]) < 1e-10
    new = pos[13].astype(np.float64) + np.array([1e-3, -2e-3, 5e-4])
    ds = C.moved_atom_sums(pos, sp, tab, qb, 13, new)
    want = mh_np.exact_delta_s(pos, sp, tab.astype(np.float64), qb, 13, new)
    assert np.abs(ds - want).max() <= 1e-9 * np.abs(want).max()
