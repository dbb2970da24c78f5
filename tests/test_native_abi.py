"""The C-ABI library builds, loads and exports every symbol of the header.

CPU-only: no compute call is made; pyiid_create must fail cleanly (status +
message, no crash) when no GB300 is present.
"""
import ctypes
import os
import re

import pytest

from conftest import REPO, gpu_available


def header_symbols():
    src = open(os.path.join(REPO, 'include', 'pyiid_gb300.h')).read()
    src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
    return sorted(set(re.findall(r'\b(pyiid_[a-z_0-9]+)\s*\(', src)))


def test_library_exports_every_header_symbol():
    from pyiid_gb300 import _native
    lib = _native.load()
    declared = header_symbols()
    assert declared, 'no symbols parsed from the header'
    for name in declared:
        assert hasattr(lib, name), f'{name} missing from the library'
    # the Python binding declares exactly the header's entry points
    assert set(_native.symbols()) == set(declared)


def test_version():
    from pyiid_gb300 import _native
    assert _native.load().pyiid_version() == 10000


@pytest.mark.skipif(gpu_available(), reason='checks the no-GPU error path')
def test_create_without_gpu_reports_error():
    from pyiid_gb300 import _native
    lib = _native.load()
    h = ctypes.c_void_p()
    rc = lib.pyiid_create(ctypes.byref(h), 0)
    assert rc != 0
    assert lib.pyiid_last_error(None)
    with pytest.raises(_native.NativeError):
        _native.Context(0)


def test_null_context_is_rejected():
    from pyiid_gb300 import _native
    lib = _native.load()
    assert lib.pyiid_set_stream(None, None) != 0
    assert lib.pyiid_synchronize(None) != 0
    assert lib.pyiid_launch_count(None) == -1


def test_variant_tables_are_described_without_a_gpu():
    """Launch-shape tables (host-only calls): counts, parameters, and the
    context's default F(Q) shape {56, -3} at index 23."""
    from pyiid_gb300 import _native
    from pyiid_gb300.autotune import variants
    lib = _native.load()
    for kern, k in _native.KERNELS.items():
        n = lib.pyiid_variant_count(k)
        assert n >= 2, kern
        v = variants(kern)
        assert [i for i, _ in v] == list(range(n))
        for _, info in v:
            assert info['bins_per_thread'] > 0 and info['threads'] > 0
    assert lib.pyiid_variant_count(99) == -1
    p = (ctypes.c_int32 * 3)()
    assert lib.pyiid_variant_info(0, 10 ** 6, p, 3) != 0
    fq = dict(variants('fq'))
    assert (fq[23]['bins_per_thread'], fq[23]['pairs_per_thread']) == (56, -3)
    for _, info in variants('fq_grad'):
        assert info['pairs_per_thread'] == 0          # packed kernels only
        assert info['threads'] % 32 == 0 and 32 % (info['threads'] // 32) == 0
    # the surrogate MLP: mma.sync, tcgen05 one tile, tcgen05 two tiles
    mlp = [(i['bins_per_thread'], i['pairs_per_thread'], i['threads'])
           for _, i in variants('mlp')]
    assert mlp == [(16, 0, 256), (128, 1, 128), (256, 1, 512)]


def header_prototypes():
    """name -> (return type text, [parameter type texts]) from the header."""
    src = open(os.path.join(REPO, 'include', 'pyiid_gb300.h')).read()
    src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
    src = re.sub(r'//[^\n]*', '', src)
    protos = {}
    for m in re.finditer(r'([A-Za-z_][\w\s\*]*?)\b(pyiid_[a-z_0-9]+)\s*\(([^)]*)\)\s*;',
                         src):
        ret, name, params = m.group(1).strip(), m.group(2), m.group(3)
        params = ' '.join(params.split())
        plist = [] if params in ('', 'void') else [p.strip()
                                                   for p in params.split(',')]
        protos[name] = (ret, plist)
    return protos


def _kind_of_c(t):
    t = t.replace('const ', '')
    if '*' in t:
        return 'ptr'
    base = t.split()[0]
    return {'int': 'i32', 'int32_t': 'i32', 'int64_t': 'i64', 'size_t': 'u64',
            'uint64_t': 'u64', 'float': 'f32', 'double': 'f64'}[base]


def _kind_of_ctypes(t):
    if t in (ctypes.c_void_p, ctypes.c_char_p) or hasattr(t, 'contents'):
        return 'ptr'
    return {ctypes.c_int: 'i32', ctypes.c_int32: 'i32', ctypes.c_int64: 'i64',
            ctypes.c_uint64: 'u64', ctypes.c_size_t: 'u64',
            ctypes.c_float: 'f32', ctypes.c_double: 'f64'}[t]


def test_binding_matches_every_prototype():
    """Every ctypes declaration in _native has the header prototype's
    argument count, and each argument and the return value the same kind
    (pointer, 32/64-bit integer, float, double): a mismatch would pass
    garbage through the C ABI without any error."""
    from pyiid_gb300 import _native
    protos = header_prototypes()
    assert set(protos) == set(_native.symbols())
    for name, (ret, params) in protos.items():
        res, args = _native._SIGNATURES[name]
        assert len(args) == len(params), (name, len(args), len(params))
        for i, (c, py) in enumerate(zip(params, args)):
            # drop the parameter name: the last identifier of the text
            ctype = re.sub(r'\b\w+$', '', c).strip() or c
            assert _kind_of_c(ctype) == _kind_of_ctypes(py), (name, i, c)
        assert _kind_of_c(ret) == _kind_of_ctypes(res), (name, ret)


def test_context_call_keeps_stream_and_call_together():
    """Threads sharing one context: every entry point runs on the stream its
    own caller set (pyiid_set_stream and the call are not interleaved).
    A fake library stands in for the device."""
    import threading
    import time
    from pyiid_gb300 import _native

    class FakeLib:
        def __init__(self):
            self.stream = None
            self.mismatch = 0

        def pyiid_set_stream(self, handle, stream):
            self.stream = stream.value
            return 0

        def pyiid_fake(self, handle, want):
            seen = self.stream
            time.sleep(0)  # give the other thread a chance to interleave
            if self.stream != want or seen != want:
                self.mismatch += 1
            return 0

    ctx = _native.Context.__new__(_native.Context)
    ctx._lib = FakeLib()
    ctx.handle = ctypes.c_void_p(1)
    ctx.device = 0
    ctx._call_lock = threading.RLock()

    def worker(s):
        for _ in range(2000):
            ctx.call('pyiid_fake', s, stream=s)

    threads = [threading.Thread(target=worker, args=(s,)) for s in (11, 22, 33)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    ctx.handle = None  # nothing to destroy
    assert ctx._lib.mismatch == 0
