"""Argument checks of the device API that run before any library call.

The C ABI receives bare pointers, so the Python layer checks what the
library will read: 3 floats per atom, one species id per atom, a 2-D
form-factor table, for packed configurations at least as many position
rows and species ids as the offsets cover, [.., 3, ..] gradients, and
gobs / gcalc as long as the r grid; host data for the transforms and
potentials is copied to the device first.  A violation raises NativeError
before any device work (here on the CPU, where no device exists)."""
import numpy as np
import pytest
import torch

from pyiid_gb300 import debye
from pyiid_gb300._native import NativeError


@pytest.mark.parametrize('shape', [(5, 3), (2, 4, 3), (3,), (0, 3)])
def test_positions_with_xyz_last_are_accepted(shape):
    assert debye._positions_shape(np.zeros(shape)) == shape
    assert debye._positions_shape(torch.zeros(shape)) == shape


@pytest.mark.parametrize('shape', [(5, 2), (15,), (3, 4), (), (0,)])
def test_positions_without_xyz_last_are_refused(shape):
    with pytest.raises(NativeError, match='positions must be'):
        debye._positions_shape(np.zeros(shape))


def test_shape_is_checked_before_the_device():
    # on a machine without a device the shape error still comes first
    with pytest.raises(NativeError, match='positions must be'):
        debye.fq(np.zeros((4, 2), np.float32), np.zeros(4, np.int32),
                 np.ones((1, 10), np.float32), 0.1)
    with pytest.raises(NativeError, match='positions must be'):
        debye.batch_fq(np.zeros(12, np.float32), np.zeros(4, np.int32),
                       [0, 4], np.ones((1, 10), np.float32), 0.1)


def test_single_configuration_species_and_table():
    tab = np.ones((2, 10), np.float32)
    debye._check_system(4, np.zeros(4, np.int32), tab)
    debye._check_system(0, np.zeros(0, np.int32), tab)
    for sp, t in ((np.zeros(3, np.int32), tab),      # too few ids
                  (np.zeros(5, np.int32), tab),      # too many ids
                  (np.zeros((4, 1), np.int32), tab),  # not 1-D
                  (np.zeros(4, np.int32), np.ones(10, np.float32))):
        with pytest.raises(NativeError, match='species must be'):
            debye._check_system(4, sp, t)


def test_packed_configurations_cover_their_buffers():
    tab = np.ones((1, 10), np.float32)
    off = np.array([0, 3, 3, 7], np.int32)
    debye._check_packed(7, np.zeros(7, np.int32), off, tab)
    # more rows than the offsets cover (capacity buffers) are fine
    debye._check_packed(9, np.zeros(9, np.int32), off, tab)
    with pytest.raises(NativeError, match='offsets cover 7 atoms'):
        debye._check_packed(6, np.zeros(7, np.int32), off, tab)
    with pytest.raises(NativeError, match='offsets cover 7 atoms'):
        debye._check_packed(7, np.zeros(6, np.int32), off, tab)
    with pytest.raises(NativeError, match='offsets cover'):
        debye._check_packed(7, np.zeros(7, np.int32), off, tab[0])
    # a decreasing last offset cannot hide a larger one
    with pytest.raises(NativeError, match='offsets cover 9 atoms'):
        debye._check_packed(7, np.zeros(7, np.int32),
                            np.array([0, 9, 5], np.int32), tab)
    with pytest.raises(NativeError, match='offsets must be'):
        debye._check_packed(7, np.zeros(7, np.int32),
                            np.array([0], np.int32), tab)


@pytest.fixture
def host_tensors(monkeypatch):
    """Runs the checks of the transform and potential calls on the CPU: the
    copy to the device is replaced by a host copy, so a call with valid
    shapes gets as far as the device context, which does not exist here."""
    def host_tensor(t, dtype, device=None):
        if not isinstance(t, torch.Tensor):
            t = torch.as_tensor(np.asarray(t))
        return t.detach().to(dtype=dtype).contiguous()
    monkeypatch.setattr(debye, '_dev_tensor', host_tensor)


def test_transform_shapes(host_tensors):
    rg = np.arange(0.0, 4.0, 0.1)
    with pytest.raises(NativeError, match='F\\(Q\\) must be'):
        debye.pdf(torch.zeros(2, 3, 4), 0.1, 0.1, rg, 0.0)
    with pytest.raises(NativeError, match='no CUDA'):
        debye.pdf(torch.zeros(2, 50), 0.1, 0.1, rg, 0.0)
    with pytest.raises(NativeError, match='gradient must be'):
        debye.grad_pdf(torch.zeros(5, 2, 50), 0.1, 0.1, rg, 0.0)
    with pytest.raises(NativeError, match='gradient must be'):
        debye.grad_pdf(torch.zeros(5, 50), 0.1, 0.1, rg, 0.0)
    with pytest.raises(NativeError, match='no CUDA'):
        debye.grad_pdf(torch.zeros(5, 3, 50), 0.1, 0.1, rg, 0.0)


def test_potential_lengths_follow_the_r_grid(host_tensors):
    r = 40
    with pytest.raises(NativeError, match='gcalc must be'):
        debye.potential(torch.zeros(r), torch.zeros(2, 2, r))
    with pytest.raises(NativeError, match=f'gobs has {r - 1} values'):
        debye.potential(torch.zeros(r - 1), torch.zeros(2, r))
    with pytest.raises(NativeError, match='no CUDA'):
        debye.potential(torch.zeros(r), torch.zeros(2, r))
    with pytest.raises(NativeError, match='grad_pdf must be'):
        debye.potential_grad(torch.zeros(5, r), torch.zeros(r),
                             torch.zeros(r))
    with pytest.raises(NativeError, match=f'gcalc has {r - 1} values'):
        debye.potential_grad(torch.zeros(5, 3, r), torch.zeros(r - 1),
                             torch.zeros(r))
    with pytest.raises(NativeError, match=f'gobs has {r + 1} values'):
        debye.potential_grad(torch.zeros(5, 3, r), torch.zeros(r),
                             torch.zeros(r + 1))
    with pytest.raises(NativeError, match='no CUDA'):
        debye.potential_grad(torch.zeros(5, 3, r), torch.zeros(r),
                             torch.zeros(r))


def test_without_a_device_host_data_is_refused_cleanly():
    # the real copy to the device raises NativeError, not a torch error
    with pytest.raises(NativeError, match='no CUDA'):
        debye.pdf(np.zeros(50, np.float32), 0.1, 0.1, np.arange(0, 4, .1), 0)


def test_surrogate_checks_its_device_buffers(monkeypatch):
    """The surrogate's kernels read descriptors [N, C] in bfloat16 on the
    device and one dL/dE per configuration of the last forward; anything
    else is refused before the library is called (a recording fake stands in
    for the device context)."""
    from pyiid_gb300 import surrogate

    calls = []

    class FakeCtx:
        def call(self, name, *args, **kw):
            calls.append(name)

    monkeypatch.setattr(surrogate, 'context', lambda index=None: FakeCtx())
    sur = surrogate.RBFMLPSurrogate(n_centres=8, n_hidden=16, device='cpu')
    off = np.array([0, 5, 9])
    with pytest.raises(NativeError, match='descriptors must be'):
        sur.forward(torch.zeros((9, 8), dtype=torch.bfloat16), off)
    with pytest.raises(NativeError, match='d_energy'):
        sur.backward(torch.zeros(2, dtype=torch.float64))  # no forward yet
    sur._last_b = 2
    with pytest.raises(NativeError, match='d_energy'):
        sur.backward(torch.zeros(3, dtype=torch.float64))
    assert calls == []
    g = sur.backward(np.array([0.5, -1.0]))   # host values are accepted
    assert calls == ['pyiid_mlp_backward'] and set(g) == set(sur.params)
