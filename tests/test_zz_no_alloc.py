"""pyiid_fq_noalloc: F(Q) for callers that cannot allocate device memory.

The entry point keeps all device-side intermediates in a fixed array inside
the library instead of allocating them.  Through the C ABI, two calls in a
row (different particles, so stale contents would show) must match pyiid_fq
within the F(Q) tolerance of the other GPU tests, and an oversized problem
must be refused with a message.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_F = 1e-5


def _run(lib, ctx, name, pos_t, sp, tab, qbin, kb):
    import torch
    out = torch.full((tab.shape[1],), float('nan'), dtype=torch.float32,
                     device='cuda')
    rc = getattr(lib, name)(
        ctx.handle, ctypes.c_void_p(pos_t.data_ptr()),
        sp.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), len(sp),
        tab.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), tab.shape[0],
        tab.shape[1], float(qbin), int(kb), ctypes.c_void_p(out.data_ptr()))
    torch.cuda.synchronize()
    return rc, out.cpu().numpy()


def test_noalloc_matches_fq_two_calls_in_a_row():
    import torch
    from pyiid_gb300 import _native, structures
    from pyiid_gb300.scatter_factors import species_tables
    lib = _native.load()
    ctx = _native.context(0)
    lib.pyiid_set_stream(ctx.handle, ctypes.c_void_p(
        torch.cuda.current_stream().cuda_stream))
    cases = [
        (structures.displaced(structures.fcc_sphere(4.08, 9.0), 0.05, 3),
         None, 0.05, 500, 2),
        (structures.random_cube(150, 12.0, 4),
         list(np.random.default_rng(4).choice([78, 79], 150)), 0.0756865, 330,
         7),
        # one 1,000-atom particle: its 32 tiles are cut into short J runs
        # (one tile pair per work item) so that the launch fills the GPU
        (structures.displaced(structures.fcc_nearest(4.08, 1000), 0.05, 4),
         None, 0.05, 500, 2),
    ]
    for pos, nums, qbin, nb, kb in cases:
        nums = nums if nums is not None else [79] * len(pos)
        sp, tab, _ = species_tables(nums, qbin, nb)
        sp = np.ascontiguousarray(sp, np.int32)
        tab = np.ascontiguousarray(tab, np.float32)
        p = torch.as_tensor(pos, device='cuda')
        rc0, want = _run(lib, ctx, 'pyiid_fq', p, sp, tab, qbin, kb)
        rc1, got = _run(lib, ctx, 'pyiid_fq_noalloc', p, sp, tab, qbin, kb)
        assert rc0 == 0 and rc1 == 0, lib.pyiid_last_error(ctx.handle)
        assert np.all(got[:kb] == 0)
        err = np.linalg.norm(got[kb:] - want[kb:]) / np.linalg.norm(want[kb:])
        assert err <= TOL_F, err


def test_noalloc_rejects_oversized_problem():
    import torch
    from pyiid_gb300 import _native, structures
    from pyiid_gb300.scatter_factors import species_tables
    lib = _native.load()
    ctx = _native.context(0)
    # 16,000 atoms x 1500 bins needs ~50 MB of partial rows (> 32 MiB)
    pos = structures.random_cube(16000, 60.0, 5)
    sp, tab, _ = species_tables([79] * 16000, 0.02, 1500)
    p = torch.as_tensor(pos, device='cuda')
    rc, _ = _run(lib, ctx, 'pyiid_fq_noalloc', p,
                 np.ascontiguousarray(sp, np.int32),
                 np.ascontiguousarray(tab, np.float32), 0.02, 25)
    assert rc == 1
    assert b'scratch' in lib.pyiid_last_error(ctx.handle)
