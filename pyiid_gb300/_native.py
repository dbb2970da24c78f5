"""ctypes binding of the C ABI in ``include/pyiid_gb300.h``.

This is the only way the package reaches the GPU.  There is no CPU fallback:
if the library is missing, fails to load, or no sm_103a device is present,
every entry point raises :class:`NativeError`.
"""
import ctypes
import os
import threading

from . import build as _build

__all__ = ['NativeError', 'load', 'symbols', 'Context', 'context',
           'PYIID_OK', 'POTENTIALS']

PYIID_OK = 0
POTENTIALS = {'rw': 0, 'chi_sq': 1}

_c_int = ctypes.c_int
_c_dbl = ctypes.c_double
_vp = ctypes.c_void_p
_i32p = ctypes.POINTER(ctypes.c_int32)
_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)

# name -> (restype, argtypes); device pointers travel as c_void_p
_SIGNATURES = {
    'pyiid_version': (_c_int, []),
    'pyiid_create': (_c_int, [ctypes.POINTER(_vp), _c_int]),
    'pyiid_destroy': (_c_int, [_vp]),
    'pyiid_set_stream': (_c_int, [_vp, _vp]),
    'pyiid_synchronize': (_c_int, [_vp]),
    'pyiid_last_error': (ctypes.c_char_p, [_vp]),
    'pyiid_launch_count': (ctypes.c_int64, [_vp]),
    'pyiid_fq': (_c_int, [_vp, _vp, _i32p, _c_int, _f32p, _c_int, _c_int,
                          _c_dbl, _c_int, _vp]),
    'pyiid_grad_fq': (_c_int, [_vp, _vp, _i32p, _c_int, _f32p, _c_int,
                               _c_int, _c_dbl, _c_int, _vp]),
    'pyiid_fq_grad': (_c_int, [_vp, _vp, _i32p, _c_int, _f32p, _c_int,
                               _c_int, _c_dbl, _c_int, _vp, _vp]),
    'pyiid_fq_grad_part': (_c_int, [_vp, _vp, _i32p, _c_int, _f32p, _c_int,
                                    _c_int, _c_dbl, _c_int, _c_int, _c_int,
                                    _vp, _vp, _i32p]),
    'pyiid_fq_from_sums': (_c_int, [_vp, _i32p, _c_int, _f32p, _c_int,
                                    _c_int, _c_int, _vp, _vp]),
    'pyiid_batch_fq': (_c_int, [_vp, _vp, _i32p, _i32p, _c_int, _f32p,
                                _c_int, _c_int, _c_dbl, _c_int, _vp]),
    'pyiid_pdf': (_c_int, [_vp, _vp, _c_int, _c_int, _c_dbl, _c_dbl, _f64p,
                           _c_int, _c_dbl, _vp]),
    'pyiid_grad_pdf': (_c_int, [_vp, _vp, _c_int, _c_int, _c_dbl, _c_dbl,
                                _f64p, _c_int, _c_dbl, _vp]),
    'pyiid_potential': (_c_int, [_vp, _vp, _vp, _c_int, _c_int, _c_int, _vp]),
    'pyiid_potential_weighted': (_c_int, [_vp, _vp, _vp, _vp, _c_int, _c_int,
                                          _vp]),
    'pyiid_potential_grad': (_c_int, [_vp, _vp, _vp, _vp, _c_int, _c_int,
                                      _c_int, _vp]),
    'pyiid_batch_potential_grad': (_c_int, [
        _vp, _vp, _i32p, _i32p, _c_int, _f32p, _c_int, _c_int, _c_dbl,
        _c_dbl, _f64p, _c_int, _c_dbl, _vp, _c_int, _vp, _vp, _vp, _vp]),
    'pyiid_mh_state_size': (ctypes.c_size_t, [_c_int, _c_int]),
    'pyiid_mh_init': (_c_int, [
        _vp, _vp, _i32p, _i32p, _c_int, _f32p, _c_int, _c_int, _c_dbl,
        _c_dbl, _f64p, _c_int, _c_dbl, _vp, _c_int, _vp, _vp]),
    'pyiid_mh_steps': (_c_int, [
        _vp, _vp, _i32p, _i32p, _c_int, _f32p, _c_int, _c_int, _c_dbl,
        _c_dbl, _f64p, _c_int, _c_dbl, _c_int, _c_dbl, _c_dbl,
        ctypes.c_float, ctypes.c_uint64, _c_int, _vp, _vp, _vp, _vp, _vp]),
    'pyiid_mc_propose': (_c_int, [
        _vp, _vp, _i32p, _i32p, _c_int, _f32p, _c_int, _c_int, _c_dbl,
        _c_dbl, _f64p, _c_int, _c_dbl, _c_int, _i32p, _i32p, _f32p, _i32p,
        _vp, _vp]),
    'pyiid_mc_accept': (_c_int, [_vp, _i32p, _c_int, _c_int, _vp, _vp, _vp]),
    'pyiid_spring': (_c_int, [_vp, _vp, _c_int, _c_dbl, _c_dbl, _c_int,
                              _f64p, _vp, _vp, _vp]),
    'pyiid_spring_voxels': (_c_int, [_vp, _vp, _c_int, _c_dbl, _c_dbl,
                                     _c_int, _f64p, _c_int, _c_int, _c_int,
                                     _c_dbl, _vp]),
    'pyiid_fq_noalloc': (_c_int, [_vp, _vp, _i32p, _c_int, _f32p, _c_int,
                                  _c_int, _c_dbl, _c_int, _vp]),
    'pyiid_rbf_features': (_c_int, [_vp, _vp, _i32p, _c_int, _c_int,
                                    ctypes.c_float, ctypes.c_float, _vp,
                                    _vp]),
    'pyiid_mlp_forward': (_c_int, [_vp, _vp, _c_int, _c_int, _i32p, _c_int,
                                   _vp, _vp, _vp, _vp, _vp, _vp, _c_int,
                                   _vp]),
    'pyiid_mlp_backward': (_c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                    _vp]),
    'pyiid_neighbor_list': (_c_int, [_vp, _vp, _i32p, _c_int, ctypes.c_float,
                                     _c_int, _vp, _vp]),
    'pyiid_surrogate_forces': (_c_int, [
        _vp, _vp, _i32p, _c_int, _vp, _vp, _c_int, _c_int, ctypes.c_float,
        ctypes.c_float, _vp, _vp, _vp, _vp, _vp, _vp, _c_int, ctypes.c_float,
        _vp, _vp, _vp]),
    'pyiid_variant_count': (_c_int, [_c_int]),
    'pyiid_variant_info': (_c_int, [_c_int, _c_int, _i32p, _c_int]),
    'pyiid_set_variant': (_c_int, [_vp, _c_int, _c_int]),
    'pyiid_get_variant': (_c_int, [_vp, _c_int]),
}

KERNELS = {'fq': 0, 'grad_fq': 1, 'adjoint': 2, 'fq_grad': 3, 'mlp': 4}


class NativeError(RuntimeError):
    """Raised when the sm_103a library cannot be used or a call fails."""


_lib = None
_lock = threading.Lock()


def load():
    """Load (building in-tree first if needed) and declare the library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.lib_path()
        # rebuild when the stamp does not match the sources (a copied or
        # checked-out library next to edited sources is never loaded); a
        # machine without nvcc loads what is there
        try:
            _build.build()
        except Exception as e:  # noqa: BLE001
            if not os.path.exists(path):
                raise NativeError(f'native library {path} is missing and '
                                  f'could not be built: {e}') from e
        try:
            lib = ctypes.CDLL(path)
        except OSError as e:
            raise NativeError(f'cannot load {path}: {e}') from e
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def symbols():
    """Names of the C entry points this binding declares."""
    return sorted(_SIGNATURES)


def _ptr(arr, ctype):
    return arr.ctypes.data_as(ctypes.POINTER(ctype))


class Context:
    """Owns one ``pyiid_ctx`` on one CUDA device."""

    def __init__(self, device=0):
        self._lib = load()
        h = _vp()
        rc = self._lib.pyiid_create(ctypes.byref(h), int(device))
        if rc != PYIID_OK:
            msg = self._lib.pyiid_last_error(None).decode()
            raise NativeError(f'pyiid_create failed ({rc}): {msg}')
        self.handle = h
        self.device = int(device)
        # set_stream + call must not interleave between threads that share
        # this context (each call runs on the stream its caller chose)
        self._call_lock = threading.RLock()

    def close(self):
        if getattr(self, 'handle', None):
            self._lib.pyiid_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass

    def check(self, rc, what):
        if rc != PYIID_OK:
            msg = self._lib.pyiid_last_error(self.handle).decode()
            raise NativeError(f'{what} failed ({rc}): {msg}')

    def call(self, name, *args, stream=None):
        """Call entry point ``name`` on the given (or torch's current) stream."""
        if stream is None:
            import torch
            stream = torch.cuda.current_stream(self.device).cuda_stream
        with self._call_lock:
            self.check(self._lib.pyiid_set_stream(self.handle, _vp(stream)),
                       'pyiid_set_stream')
            self.check(getattr(self._lib, name)(self.handle, *args), name)

    def synchronize(self):
        self.check(self._lib.pyiid_synchronize(self.handle),
                   'pyiid_synchronize')

    def set_variant(self, kernel, variant):
        self.check(self._lib.pyiid_set_variant(self.handle, KERNELS[kernel],
                                               int(variant)),
                   'pyiid_set_variant')

    def get_variant(self, kernel):
        return int(self._lib.pyiid_get_variant(self.handle, KERNELS[kernel]))

    @property
    def launches(self):
        return int(self._lib.pyiid_launch_count(self.handle))


_contexts = {}


def context(device=None):
    """The per-device shared :class:`Context` (created on first use)."""
    import torch
    if not torch.cuda.is_available():
        raise NativeError('no CUDA device is visible; pyiid_gb300 runs only '
                          'on a GB300 (sm_103a) GPU')
    dev = torch.cuda.current_device() if device is None else int(device)
    with _lock:
        ctx = _contexts.get(dev)
    if ctx is None:
        ctx = Context(dev)
        with _lock:
            _contexts[dev] = ctx
    return ctx
