"""Device-side functional API over the C ABI (torch tensors in, tensors out).

Inputs that describe the system (species ids, form-factor tables, r grid) are
host numpy arrays; positions, F(Q), G(r) and gradients are CUDA tensors on the
current device, so chains of calls stay on the GPU.  Every function launches
on torch's current stream.
"""
import numpy as np
import torch

from ._native import context, POTENTIALS, NativeError

__all__ = ['fq', 'batch_fq', 'grad_fq', 'fq_grad', 'fq_grad_part',
           'fq_from_sums', 'pdf', 'grad_pdf', 'potential', 'potential_grad',
           'batch_potential_grad', 'as_positions', 'mh_init', 'mh_steps',
           'mh_state_size', 'mh_views', 'mc_propose', 'mc_accept',
           'MOVE_DISPLACE', 'MOVE_INSERT', 'MOVE_REMOVE']

MOVE_DISPLACE, MOVE_INSERT, MOVE_REMOVE = 0, 1, 2

_f32p = None


def _np(a, dtype):
    return np.ascontiguousarray(np.asarray(a, dtype=dtype))


def _ptr(a, ctype):
    import ctypes
    return a.ctypes.data_as(ctypes.POINTER(ctype))


_cuda_seen = False


def _positions_shape(x):
    """Shape of positions given as a tensor, an array or nested lists; the
    last axis must hold x, y, z (the kernels read 3 floats per atom)."""
    shape = tuple(x.shape) if hasattr(x, 'shape') else np.shape(x)
    if len(shape) == 0 or shape[-1] != 3:
        raise NativeError(f'positions must be [N, 3] (got {list(shape)})')
    return shape


def _check_system(n, sp, tab):
    """One configuration: species ids [n] and a form-factor table [S, K]
    (the library reads n ids and S x K floats from these host arrays)."""
    if tab.ndim != 2 or sp.ndim != 1 or sp.shape[0] != n:
        raise NativeError(f'species must be [{n}] and scatter [S, K] (got '
                          f'{list(sp.shape)} and {list(tab.shape)})')


def _check_packed(n_rows, sp, off, tab):
    """Packed configurations: offsets [B+1] and at least offsets' atoms of
    positions (n_rows) and species ids (the library reads that many)."""
    if off.ndim != 1 or off.shape[0] < 2:
        raise NativeError('offsets must be [B + 1] with B >= 1')
    total = int(off.max())
    if tab.ndim != 2 or sp.ndim != 1 or sp.shape[0] < total or \
            n_rows < total:
        raise NativeError(f'offsets cover {total} atoms: positions has '
                          f'{n_rows} rows, species {list(sp.shape)}, '
                          f'scatter must be [S, K] (got {list(tab.shape)})')


def _require_cuda():
    global _cuda_seen
    if not _cuda_seen:  # a device, once seen, stays (the check costs µs)
        if not torch.cuda.is_available():
            raise NativeError('no CUDA device is visible; pyiid_gb300 runs '
                              'only on a GB300 (sm_103a) GPU')
        _cuda_seen = True


def _dev_tensor(t, dtype, device=None):
    """Contiguous CUDA tensor of ``dtype`` from a tensor or an array.  Host
    data is copied to the device: the library dereferences device
    pointers only."""
    _require_cuda()
    if not isinstance(t, torch.Tensor):
        t = torch.as_tensor(np.asarray(t))
    t = t.detach()
    if device is None:
        device = t.device if t.is_cuda else torch.device('cuda')
    return t.to(device=device, dtype=dtype).contiguous()


def _check_len(t, n, name):
    if t.numel() != n:
        raise NativeError(f'{name} has {t.numel()} values, expected {n}')


def as_positions(x, device=None):
    """float32 contiguous CUDA tensor [N, 3] from an array or tensor (any
    leading shape with x, y, z last, e.g. [B, N, 3], is flattened)."""
    _positions_shape(x)
    _require_cuda()
    if isinstance(x, torch.Tensor):
        t = x.detach()
        if not t.is_cuda:
            t = t.to('cuda' if device is None else device)
        return t.to(torch.float32).contiguous().reshape(-1, 3)
    return torch.as_tensor(_np(x, np.float32),
                           device=device or 'cuda').reshape(-1, 3)


def _check_dev(t, name, dtype):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise NativeError(f'{name} must be a CUDA tensor')
    if t.dtype != dtype or not t.is_contiguous():
        raise NativeError(f'{name} must be a contiguous {dtype} tensor')


def _check_out(t, name, dtype):
    """An output the device can write: a CUDA tensor, or a pinned CPU tensor
    (written in place by the kernel over the host link)."""
    if isinstance(t, torch.Tensor) and not t.is_cuda and t.is_pinned():
        if t.dtype != dtype or not t.is_contiguous():
            raise NativeError(f'{name} must be a contiguous {dtype} tensor')
        return
    _check_dev(t, name, dtype)


def fq(positions, species, scatter, qbin, k_begin=0, out=None):
    """Reduced structure factor [K] (bins from Q = 0; bins < k_begin are 0).

    The value of the reference processor callable ``self.fq`` before the
    getter slices it (wrap_fq, pyiid/experiments/elasticscatter/
    cpu_wrappers/flat_multi_cpu_wrap.py:22-60).
    """
    import ctypes
    pos = as_positions(positions)
    n = pos.shape[0]
    sp = _np(species, np.int32)
    tab = _np(scatter, np.float32)
    _check_system(n, sp, tab)
    if out is None:
        out = torch.empty(tab.shape[1], dtype=torch.float32, device=pos.device)
    else:
        _check_dev(out, 'out', torch.float32)
        _check_len(out, tab.shape[1], 'out')
    ctx = context(pos.device.index)
    ctx.call('pyiid_fq', ctypes.c_void_p(pos.data_ptr()),
             _ptr(sp, ctypes.c_int32), n, _ptr(tab, ctypes.c_float),
             tab.shape[0], tab.shape[1], float(qbin), int(k_begin),
             ctypes.c_void_p(out.data_ptr()))
    return out


def batch_fq(positions, species, offsets, scatter, qbin, k_begin=0,
             out=None):
    """F(Q) rows [B, K] of packed configurations (offsets [B+1])."""
    import ctypes
    pos = as_positions(positions)
    sp = _np(species, np.int32)
    off = _np(offsets, np.int32)
    tab = _np(scatter, np.float32)
    _check_packed(pos.numel() // 3, sp, off, tab)
    b = len(off) - 1
    if out is None:
        out = torch.empty((b, tab.shape[1]), dtype=torch.float32,
                          device=pos.device)
    else:
        _check_dev(out, 'out', torch.float32)
        _check_len(out, b * tab.shape[1], 'out')
    ctx = context(pos.device.index)
    ctx.call('pyiid_batch_fq', ctypes.c_void_p(pos.data_ptr()),
             _ptr(sp, ctypes.c_int32), _ptr(off, ctypes.c_int32), b,
             _ptr(tab, ctypes.c_float), tab.shape[0], tab.shape[1],
             float(qbin), int(k_begin), ctypes.c_void_p(out.data_ptr()))
    return out


def grad_fq(positions, species, scatter, qbin, k_begin=0, out=None):
    """Reference-convention gradient [N, 3, K] (= -1/2 dF/dx).  Every element
    of ``out`` is written (bins < k_begin with 0).

    The value of ``self.grad`` (wrap_fq_grad, cpu_wrappers/
    flat_multi_cpu_wrap.py:63-102 of pyiid/experiments/elasticscatter).
    """
    import ctypes
    pos = as_positions(positions)
    n = pos.shape[0]
    sp = _np(species, np.int32)
    tab = _np(scatter, np.float32)
    _check_system(n, sp, tab)
    if out is None:
        out = torch.empty((n, 3, tab.shape[1]), dtype=torch.float32,
                          device=pos.device)
    else:
        _check_dev(out, 'out', torch.float32)
        _check_len(out, n * 3 * tab.shape[1], 'out')
    if n == 0:
        return out
    ctx = context(pos.device.index)
    ctx.call('pyiid_grad_fq', ctypes.c_void_p(pos.data_ptr()),
             _ptr(sp, ctypes.c_int32), n, _ptr(tab, ctypes.c_float),
             tab.shape[0], tab.shape[1], float(qbin), int(k_begin),
             ctypes.c_void_p(out.data_ptr()))
    return out


def fq_grad(positions, species, scatter, qbin, k_begin=0, out_fq=None,
            out_grad=None):
    """F(Q) [K] and the reference-convention gradient [N, 3, K] from one
    pass over the pairs (pyiid_fq_grad): the values fq() and grad_fq()
    return, with the pair terms summed in another order.  ``out_fq`` and
    ``out_grad`` may be pinned CPU tensors: the kernel then writes the
    results into host memory directly (no device-to-host copy; synchronise
    the stream before reading them)."""
    import ctypes
    pos = as_positions(positions)
    n = pos.shape[0]
    sp = _np(species, np.int32)
    tab = _np(scatter, np.float32)
    _check_system(n, sp, tab)
    k = tab.shape[1]
    if out_fq is None:
        out_fq = torch.empty(k, dtype=torch.float32, device=pos.device)
    else:
        _check_out(out_fq, 'out_fq', torch.float32)
        if out_fq.numel() != k:
            raise NativeError(f'out_fq must hold {k} floats')
    if out_grad is None:
        out_grad = torch.empty((n, 3, k), dtype=torch.float32,
                               device=pos.device)
    else:
        _check_out(out_grad, 'out_grad', torch.float32)
        if out_grad.numel() != n * 3 * k:
            raise NativeError(f'out_grad must hold {n} x 3 x {k} floats')
    ctx = context(pos.device.index)
    ctx.call('pyiid_fq_grad', ctypes.c_void_p(pos.data_ptr()),
             _ptr(sp, ctypes.c_int32), n, _ptr(tab, ctypes.c_float),
             tab.shape[0], k, float(qbin), int(k_begin),
             ctypes.c_void_p(out_fq.data_ptr()),
             ctypes.c_void_p(out_grad.data_ptr()))
    return out_fq, out_grad


def fq_grad_part(positions, species, scatter, qbin, k_begin, part, n_parts,
                 out_grad=None):
    """One part of a configuration split across processes
    (pyiid_fq_grad_part): (raw sums S_k [K] float64, gradient [N, 3, K] with
    this part's rows written, bool mask [N] of those rows).  ``out_grad`` is
    written only in this part's rows; a new one starts as zeros."""
    import ctypes
    pos = as_positions(positions)
    n = pos.shape[0]
    sp = _np(species, np.int32)
    tab = _np(scatter, np.float32)
    _check_system(n, sp, tab)
    k = tab.shape[1]
    if out_grad is None:
        out_grad = torch.zeros((n, 3, k), dtype=torch.float32,
                               device=pos.device)
    else:
        _check_dev(out_grad, 'out_grad', torch.float32)
        if out_grad.numel() != n * 3 * k:
            raise NativeError(f'out_grad must hold {n} x 3 x {k} floats')
    sums = torch.empty(k, dtype=torch.float64, device=pos.device)
    rows = np.zeros(max(n, 1), np.int32)
    ctx = context(pos.device.index)
    ctx.call('pyiid_fq_grad_part', ctypes.c_void_p(pos.data_ptr()),
             _ptr(sp, ctypes.c_int32), n, _ptr(tab, ctypes.c_float),
             tab.shape[0], k, float(qbin), int(k_begin), int(part),
             int(n_parts), ctypes.c_void_p(sums.data_ptr()),
             ctypes.c_void_p(out_grad.data_ptr()), _ptr(rows, ctypes.c_int32))
    return sums, out_grad, rows[:n].astype(bool)


def fq_from_sums(species, scatter, k_begin, sums):
    """F(Q) [K] from the raw sums of all parts (pyiid_fq_from_sums)."""
    import ctypes
    sp = _np(species, np.int32)
    tab = _np(scatter, np.float32)
    k = tab.shape[1]
    _check_dev(sums, 'sums', torch.float64)
    if sums.numel() != k:
        raise NativeError(f'sums must hold {k} doubles')
    out = torch.empty(k, dtype=torch.float32, device=sums.device)
    ctx = context(sums.device.index)
    ctx.call('pyiid_fq_from_sums', _ptr(sp, ctypes.c_int32), len(sp),
             _ptr(tab, ctypes.c_float), tab.shape[0], k, int(k_begin),
             ctypes.c_void_p(sums.data_ptr()), ctypes.c_void_p(out.data_ptr()))
    return out


def pdf(fq_t, qstep, rstep, rgrid, qmin):
    """G(r) [B, R] (float64) for F(Q) rows [B, K] (or [K] -> [R]).

    get_pdf_at_qmin (pyiid/experiments/elasticscatter/kernels/
    master_kernel.py:39-105) as one linear map per grid.
    """
    import ctypes
    f = _dev_tensor(fq_t, torch.float32)
    squeeze = f.dim() == 1
    f = f.reshape(1, -1) if squeeze else f
    if f.dim() != 2:
        raise NativeError(f'F(Q) must be [B, K] or [K] (got {list(f.shape)})')
    rg = _np(rgrid, np.float64)
    out = torch.empty((f.shape[0], len(rg)), dtype=torch.float64,
                      device=f.device)
    if len(rg):
        ctx = context(f.device.index)
        ctx.call('pyiid_pdf', ctypes.c_void_p(f.data_ptr()), f.shape[0],
                 f.shape[1], float(qstep), float(rstep),
                 _ptr(rg, ctypes.c_double), len(rg), float(qmin),
                 ctypes.c_void_p(out.data_ptr()))
    return out[0] if squeeze else out


def grad_pdf(grad_fq_t, qstep, rstep, rgrid, qmin):
    """Transform of every row of a [N, 3, K] gradient -> [N, 3, R] float64
    (grad_pdf, kernels/master_kernel.py:272-290)."""
    import ctypes
    g = _dev_tensor(grad_fq_t, torch.float32)
    if g.dim() != 3 or g.shape[1] != 3:
        raise NativeError(f'the gradient must be [N, 3, K] (got '
                          f'{list(g.shape)})')
    n, _, k = g.shape
    rg = _np(rgrid, np.float64)
    # every element is written by the kernel (a zero fill cost 15 us of the
    # 0.18 ms call at N = 1000)
    out = torch.empty((n, 3, len(rg)), dtype=torch.float64, device=g.device)
    if n and len(rg):
        ctx = context(g.device.index)
        ctx.call('pyiid_grad_pdf', ctypes.c_void_p(g.data_ptr()), n, k,
                 float(qstep), float(rstep), _ptr(rg, ctypes.c_double),
                 len(rg), float(qmin), ctypes.c_void_p(out.data_ptr()))
    return out


def potential(gobs, gcalc, kind='rw', weight=None):
    """(value, scale) rows [B, 2] for gcalc [B, R] (or [R] -> [2]): get_rw /
    get_chi_sq with get_scale (kernels/master_kernel.py:206-266, 388-389).
    ``weight`` ([R], Rw only): get_rw's per-point weights (the scale stays
    unweighted, as in the reference)."""
    import ctypes
    gc = _dev_tensor(gcalc, torch.float64)
    squeeze = gc.dim() == 1
    gc = gc.reshape(1, -1) if squeeze else gc
    if gc.dim() != 2:
        raise NativeError(f'gcalc must be [B, R] or [R] (got '
                          f'{list(gc.shape)})')
    go = _dev_tensor(gobs, torch.float64, gc.device)
    _check_len(go, gc.shape[1], 'gobs')
    out = torch.empty((gc.shape[0], 2), dtype=torch.float64, device=gc.device)
    ctx = context(gc.device.index)
    if weight is not None:
        if kind != 'rw':
            raise NativeError('weights apply to Rw only (the reference\'s '
                              'get_chi_sq takes none)')
        w = _dev_tensor(weight, torch.float64, gc.device)
        _check_len(w, gc.shape[1], 'weight')
        ctx.call('pyiid_potential_weighted', ctypes.c_void_p(go.data_ptr()),
                 ctypes.c_void_p(gc.data_ptr()), ctypes.c_void_p(w.data_ptr()),
                 gc.shape[0], gc.shape[1], ctypes.c_void_p(out.data_ptr()))
    else:
        ctx.call('pyiid_potential', ctypes.c_void_p(go.data_ptr()),
                 ctypes.c_void_p(gc.data_ptr()), gc.shape[0], gc.shape[1],
                 POTENTIALS[kind], ctypes.c_void_p(out.data_ptr()))
    return out[0] if squeeze else out


def potential_grad(grad_pdf_t, gcalc, gobs, kind='rw'):
    """sum_r c_r dG_r for each [a, c] row of grad_pdf [N, 3, R] -> [N, 3]:
    get_grad_rw / get_grad_chi_sq (kernels/master_kernel.py:293-376)."""
    import ctypes
    gp = _dev_tensor(grad_pdf_t, torch.float64)
    if gp.dim() != 3 or gp.shape[1] != 3:
        raise NativeError(f'grad_pdf must be [N, 3, R] (got '
                          f'{list(gp.shape)})')
    gc = _dev_tensor(gcalc, torch.float64, gp.device)
    go = _dev_tensor(gobs, torch.float64, gp.device)
    _check_len(gc, gp.shape[2], 'gcalc')
    _check_len(go, gp.shape[2], 'gobs')
    n = gp.shape[0]
    out = torch.zeros((n, 3), dtype=torch.float64, device=gp.device)
    if n:
        ctx = context(gp.device.index)
        ctx.call('pyiid_potential_grad', ctypes.c_void_p(gp.data_ptr()),
                 ctypes.c_void_p(gc.data_ptr()), ctypes.c_void_p(go.data_ptr()),
                 n, gp.shape[2], POTENTIALS[kind],
                 ctypes.c_void_p(out.data_ptr()))
    return out


def batch_potential_grad(positions, species, offsets, scatter, qstep, rstep,
                         rgrid, qmin, gobs, kind='rw', want_grad=True,
                         out=None):
    """Fused F -> G -> potential (+ adjoint gradient) for packed configs:
    the energy and gradient chain of Calc1D (pyiid/calc/calc_1d.py:44-95,
    wrap_rw / wrap_grad_rw in pyiid/calc/__init__.py:10-105) for many
    configurations in one call.

    positions [sum N, 3] (CUDA), species [sum N] and offsets [B+1] (host).
    Returns dict(energy [B, 2] f64, grad [sum N, 3] f32 or None,
    gcalc [B, R] f64, fq [B, K] f32).  ``out`` may pass preallocated tensors
    with those keys (used under CUDA-graph capture).
    """
    import ctypes
    pos = as_positions(positions)
    sp = _np(species, np.int32)
    off = _np(offsets, np.int32)
    tab = _np(scatter, np.float32)
    _check_packed(pos.numel() // 3, sp, off, tab)
    rg = _np(rgrid, np.float64)
    b = len(off) - 1
    dev = pos.device
    go = _dev_tensor(gobs, torch.float64, dev)
    _check_len(go, len(rg), 'gobs')
    if out is None:
        out = {
            'energy': torch.empty((b, 2), dtype=torch.float64, device=dev),
            'grad': (torch.empty((pos.shape[0], 3), dtype=torch.float32,
                                 device=dev) if want_grad else None),
            'gcalc': torch.empty((b, len(rg)), dtype=torch.float64,
                                 device=dev),
            'fq': torch.empty((b, tab.shape[1]), dtype=torch.float32,
                              device=dev),
        }
    else:
        for key, dt, size in (('energy', torch.float64, 2 * b),
                              ('gcalc', torch.float64, b * len(rg)),
                              ('fq', torch.float32, b * tab.shape[1])):
            _check_dev(out[key], key, dt)
            _check_len(out[key], size, key)
        if want_grad and out.get('grad') is not None:
            _check_dev(out['grad'], 'grad', torch.float32)
            if out['grad'].numel() < 3 * int(off.max()):
                raise NativeError(f'grad has {out["grad"].numel()} values, '
                                  f'the offsets cover {int(off.max())} atoms')
    ctx = context(dev.index)
    g = out.get('grad') if want_grad else None
    ctx.call('pyiid_batch_potential_grad', ctypes.c_void_p(pos.data_ptr()),
             _ptr(sp, ctypes.c_int32), _ptr(off, ctypes.c_int32), b,
             _ptr(tab, ctypes.c_float), tab.shape[0], tab.shape[1],
             float(qstep), float(rstep), _ptr(rg, ctypes.c_double), len(rg),
             float(qmin), ctypes.c_void_p(go.data_ptr()), POTENTIALS[kind],
             ctypes.c_void_p(out['energy'].data_ptr()),
             ctypes.c_void_p(g.data_ptr() if g is not None else 0),
             ctypes.c_void_p(out['gcalc'].data_ptr()),
             ctypes.c_void_p(out['fq'].data_ptr()))
    return out


def mh_state_size(n_configs, n_bins):
    """Doubles of the single-atom Metropolis chain state."""
    from ._native import load
    return int(load().pyiid_mh_state_size(int(n_configs), int(n_bins)))


def mh_views(state):
    """Views of the chain state buffer (layout of pyiid_mh_state_size):
    v [K], goo, S2 / F2 [2, B, K] (both buffers), uqe [B, 4] (u = G.gobs,
    q = G.G, ee = |gobs - s G|^2, 0), cur [B] (int32), and S / F [B, K]:
    each chain's current buffer (gathered copies)."""
    buf, b, k = state['buf'], state['n_configs'], state['n_bins']
    bk = b * k
    o = k + 2
    s2 = buf[o:o + 2 * bk].view(2, b, k)
    uqe = buf[o + 2 * bk:o + 2 * bk + 4 * b].view(b, 4)
    f_off = o + 2 * bk + 4 * b
    f2 = buf[f_off:f_off + bk].view(torch.float32).view(2, b, k)
    cur = buf[f_off + bk:].view(torch.int32)[:b]
    idx = cur.long()
    ar = torch.arange(b, device=buf.device)
    return {'v': buf[:k], 'goo': buf[k], 'S2': s2, 'F2': f2, 'uqe': uqe,
            'cur': cur, 'S': s2[idx, ar], 'F': f2[idx, ar]}


def mh_init(positions, species, offsets, scatter, qstep, rstep, rgrid, qmin,
            gobs, kind='rw', state=None):
    """Full exact evaluation that starts (or re-synchronises) single-atom
    Metropolis chains.  Returns (and fills) the state dict: 'buf' (the
    device chain state), 'energy' [B, 2] f64 (potential, scale),
    'n_configs', 'n_bins'."""
    import ctypes
    pos = as_positions(positions)
    sp = _np(species, np.int32)
    off = _np(offsets, np.int32)
    tab = _np(scatter, np.float32)
    _check_packed(pos.numel() // 3, sp, off, tab)
    rg = _np(rgrid, np.float64)
    b = len(off) - 1
    k = tab.shape[1]
    dev = pos.device
    go = _dev_tensor(gobs, torch.float64, dev)
    _check_len(go, len(rg), 'gobs')
    if state is None:
        state = {}
    if state.get('buf') is None or state.get('n_configs') != b or \
            state.get('n_bins') != k:
        state['buf'] = torch.zeros(mh_state_size(b, k), dtype=torch.float64,
                                   device=dev)
        state['n_configs'], state['n_bins'] = b, k
    if state.get('energy') is None:
        state['energy'] = torch.empty((b, 2), dtype=torch.float64, device=dev)
    ctx = context(dev.index)
    ctx.call('pyiid_mh_init', ctypes.c_void_p(pos.data_ptr()),
             _ptr(sp, ctypes.c_int32), _ptr(off, ctypes.c_int32), b,
             _ptr(tab, ctypes.c_float), tab.shape[0], k,
             float(qstep), float(rstep), _ptr(rg, ctypes.c_double), len(rg),
             float(qmin), ctypes.c_void_p(go.data_ptr()), POTENTIALS[kind],
             ctypes.c_void_p(state['buf'].data_ptr()),
             ctypes.c_void_p(state['energy'].data_ptr()))
    return state


def mh_steps(positions, species, offsets, scatter, qstep, rstep, rgrid, qmin,
             state, n_steps, conv, kT, sigma, seed, kind='rw', trace=None):
    """Enqueue n_steps single-atom Metropolis steps of every chain.

    positions [sum N, 3] f32 CUDA tensor, updated in place.  ``state`` is
    the dict of mh_init; 'counter' (proposals per chain) and 'accepted'
    (int64 tensors) are added if missing.  ``trace`` may be a float64 CUDA
    tensor [n_steps, B, 8] receiving every proposal (atom, x', y', z',
    log u, V', accepted, V)."""
    import ctypes
    pos = positions
    if not (isinstance(pos, torch.Tensor) and pos.is_cuda and
            pos.dtype == torch.float32 and pos.is_contiguous()):
        raise NativeError('positions must be a contiguous float32 CUDA tensor '
                          '(updated in place)')
    _positions_shape(pos)
    sp = _np(species, np.int32)
    off = _np(offsets, np.int32)
    tab = _np(scatter, np.float32)
    _check_packed(pos.numel() // 3, sp, off, tab)
    rg = _np(rgrid, np.float64)
    b = len(off) - 1
    dev = pos.device
    if state.get('n_configs') != b or state.get('n_bins') != tab.shape[1]:
        raise NativeError('state does not match the batch (call mh_init)')
    for key in ('counter', 'accepted'):
        if state.get(key) is None:
            state[key] = torch.zeros(b, dtype=torch.int64, device=dev)
    if trace is not None:
        _check_dev(trace, 'trace', torch.float64)
        if trace.numel() < n_steps * b * 8:
            raise NativeError('trace must hold n_steps * B * 8 values')
    ctx = context(dev.index)
    ctx.call('pyiid_mh_steps', ctypes.c_void_p(pos.data_ptr()),
             _ptr(sp, ctypes.c_int32), _ptr(off, ctypes.c_int32), b,
             _ptr(tab, ctypes.c_float), tab.shape[0], tab.shape[1],
             float(qstep), float(rstep), _ptr(rg, ctypes.c_double), len(rg),
             float(qmin), POTENTIALS[kind], float(conv), float(kT),
             float(sigma), int(seed) & 0xFFFFFFFFFFFFFFFF, int(n_steps),
             ctypes.c_void_p(state['buf'].data_ptr()),
             ctypes.c_void_p(state['energy'].data_ptr()),
             ctypes.c_void_p(state['counter'].data_ptr()),
             ctypes.c_void_p(state['accepted'].data_ptr()),
             ctypes.c_void_p(trace.data_ptr() if trace is not None else 0))
    return state


def mc_propose(positions, species, offsets, scatter, qstep, rstep, rgrid,
               qmin, state, mode, atom, xyz, new_species=None, kind='rw'):
    """Exact potential of one host-chosen move per chain (no state change).

    mode [B] (MOVE_DISPLACE, MOVE_INSERT, MOVE_REMOVE), atom [B] (index
    within its configuration), xyz [B, 3] (new position), new_species [B]
    (inserted species id).  Returns the device tensor eval [B, 8]:
    V', scale, u', q', ee', V (0), 0, 0; the proposal is kept in the state's
    spare buffers for :func:`mc_accept`."""
    import ctypes
    pos = as_positions(positions)
    sp = _np(species, np.int32)
    off = _np(offsets, np.int32)
    tab = _np(scatter, np.float32)
    _check_packed(pos.numel() // 3, sp, off, tab)
    rg = _np(rgrid, np.float64)
    b = len(off) - 1
    md = _np(mode, np.int32).reshape(b)
    at = _np(atom, np.int32).reshape(b)
    xz = _np(xyz, np.float32).reshape(b, 3)
    ns = _np(np.zeros(b) if new_species is None else new_species,
             np.int32).reshape(b)
    if state.get('n_configs') != b or state.get('n_bins') != tab.shape[1]:
        raise NativeError('state does not match the batch (call mh_init)')
    if state.get('eval') is None:
        state['eval'] = torch.empty((b, 8), dtype=torch.float64,
                                    device=pos.device)
    ctx = context(pos.device.index)
    ctx.call('pyiid_mc_propose', ctypes.c_void_p(pos.data_ptr()),
             _ptr(sp, ctypes.c_int32), _ptr(off, ctypes.c_int32), b,
             _ptr(tab, ctypes.c_float), tab.shape[0], tab.shape[1],
             float(qstep), float(rstep), _ptr(rg, ctypes.c_double), len(rg),
             float(qmin), POTENTIALS[kind], _ptr(md, ctypes.c_int32),
             _ptr(at, ctypes.c_int32), _ptr(xz, ctypes.c_float),
             _ptr(ns, ctypes.c_int32), ctypes.c_void_p(state['buf'].data_ptr()),
             ctypes.c_void_p(state['eval'].data_ptr()))
    return state['eval']


def mc_accept(state, accept):
    """Make the proposals of the last :func:`mc_propose` the state of the
    chains with accept[c] true (the caller then applies the moves to its
    positions, species and offsets)."""
    import ctypes
    acc = _np(np.asarray(accept, bool).astype(np.int32), np.int32)
    b = state['n_configs']
    if acc.size != b:
        raise NativeError(f'accept has {acc.size} entries, the state {b}')
    ctx = context(state['buf'].device.index)
    ctx.call('pyiid_mc_accept', _ptr(acc, ctypes.c_int32), b,
             state['n_bins'], ctypes.c_void_p(state['eval'].data_ptr()),
             ctypes.c_void_p(state['buf'].data_ptr()),
             ctypes.c_void_p(state['energy'].data_ptr()))
    return state
