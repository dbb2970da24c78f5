"""The F(Q) -> G(r) maps on the GPU against the oracle's T matrix: the
compat gradient transform (pyiid_grad_pdf: operands scaled by powers of
two and split into two FP16 halves, three tcgen05 kind::f16 products with
FP32 accumulation in tensor memory, FP64 output) over several output tiles
and both tile widths (few rows: 128 columns; many: 256), n_r even or odd
(paired or single FP64 stores), K not a multiple of the 64-bin k step,
qmin > 0 (rows below kmin skipped), qmin above the whole Q range (an
all-zero product) and rows of magnitudes 1e-30 .. 1e+30 (per-row scales);
and the batched forward transform (pyiid_pdf).
Tolerance: norm-wise relative 1e-5 (~1.2e-6 measured: 22-bit halves and
FP32 sums of K terms); per row 1e-5 of the row's norm."""
import numpy as np
import pytest
import torch

from oracle import debye_np as O

pytestmark = pytest.mark.gpu

TOL = 1e-5


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope='module')
def D():
    from pyiid_gb300 import debye
    return debye


@pytest.mark.parametrize('n,k,n_r,qmin', [(150, 333, 4001, 0.4),
                                          (43, 330, 4000, 0.0),
                                          (1, 17, 130, 0.0),
                                          (200, 64, 257, 1.0),
                                          (5, 17, 130, 1.4),
                                          (1000, 330, 4000, 0.0),
                                          (1001, 331, 3999, 0.5)])
def test_grad_pdf_matches_oracle(D, n, k, n_r, qmin):
    rng = np.random.default_rng(n + k)
    g = rng.standard_normal((n, 3, k)).astype(np.float32)
    qstep, rstep = 0.0756865, 0.01
    rg = np.arange(n_r) * rstep
    got = D.grad_pdf(torch.as_tensor(g, device='cuda'), qstep, rstep, rg,
                     qmin).cpu().numpy()
    # no bounded wait of the tensor-core pipeline gave up
    from pyiid_gb300._native import context
    context().synchronize()
    want = O.grad_pdf(g, rstep, qstep, rg, qmin)
    assert got.shape == (n, 3, n_r)
    if not np.any(want):
        assert not np.any(got)
        return
    assert rel(got, want) <= TOL, rel(got, want)


def test_grad_pdf_rows_of_very_different_magnitude(D):
    """Each row of grad_fq is scaled by its own power of two before the FP16
    split: rows from 1e-30 to 1e+30 (and an all-zero row) keep the relative
    accuracy of a row of order one."""
    rng = np.random.default_rng(11)
    n, k, n_r = 61, 330, 4000
    g = rng.standard_normal((n, 3, k))
    mags = 10.0 ** np.linspace(-30, 30, n)
    g = (g * mags[:, None, None]).astype(np.float32)
    g[7] = 0.0
    qstep, rstep = 0.0756865, 0.01
    rg = np.arange(n_r) * rstep
    got = D.grad_pdf(torch.as_tensor(g, device='cuda'), qstep, rstep, rg,
                     0.0).cpu().numpy()
    want = O.grad_pdf(g, rstep, qstep, rg, 0.0)
    assert not np.any(got[7])
    for a in range(n):
        if a == 7:
            continue
        e = np.linalg.norm(got[a] - want[a]) / np.linalg.norm(want[a])
        assert e <= TOL, (a, mags[a], e)


@pytest.mark.parametrize('b,k,n_r,qmin', [(64, 330, 4000, 0.0),
                                          (3, 333, 4001, 0.5)])
def test_batched_pdf_matches_oracle(D, b, k, n_r, qmin):
    rng = np.random.default_rng(b)
    f = rng.standard_normal((b, k)).astype(np.float32)
    qstep, rstep = 0.0756865, 0.01
    rg = np.arange(n_r) * rstep
    got = D.pdf(torch.as_tensor(f, device='cuda'), qstep, rstep, rg,
                qmin).cpu().numpy()
    T = O.tmatrix(k, rstep, qstep, rg, qmin)
    want = f.astype(np.float64) @ T
    assert rel(got, want) <= TOL, rel(got, want)


def test_grad_pdf_into_an_output_at_an_odd_offset(D):
    """The compat gradient GEMM writing rows that start 8 bytes past a
    16-byte boundary takes its scalar stores and equals the aligned call."""
    import ctypes
    from pyiid_gb300._native import context
    n, k, n_r = 20, 330, 400
    rng = np.random.default_rng(3)
    g = torch.as_tensor(rng.standard_normal((n, 3, k)).astype(np.float32),
                        device='cuda')
    qstep, rstep = 0.0756865, 0.01
    rg = np.arange(n_r) * rstep
    want = D.grad_pdf(g, qstep, rstep, rg, 0.0)
    big = torch.full((n * 3 * n_r + 2,), float('nan'), dtype=torch.float64,
                     device='cuda')
    ptr = big.data_ptr() + 8
    assert ptr % 16 == 8
    rgc = np.ascontiguousarray(rg, np.float64)
    context().call('pyiid_grad_pdf', ctypes.c_void_p(g.data_ptr()), n, k,
                   float(qstep), float(rstep),
                   rgc.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), n_r,
                   0.0, ctypes.c_void_p(ptr))
    got = big[1:1 + n * 3 * n_r].view(n, 3, n_r)
    assert torch.equal(got, want)
    assert torch.isnan(big[0]) and torch.isnan(big[-1])
