"""Configuration sharding on two CPU ranks (gloo, 127.0.0.1): balanced
contiguous slices, per-rank evaluation of the slice, order-preserving
gather and max-over-ranks timing."""
import os
import socket

import numpy as np
import pytest

from pyiid_gb300.distributed import pair_costs, shard_bounds


def test_shard_bounds_cover_and_balance():
    rng = np.random.default_rng(0)
    sizes = rng.integers(55, 2001, 256)
    offsets = np.concatenate([[0], np.cumsum(sizes)])
    costs = pair_costs(offsets)
    for world in (1, 2, 3, 8):
        b = shard_bounds(costs, world)
        assert b[0][0] == 0 and b[-1][1] == len(sizes)
        assert all(b[r][1] == b[r + 1][0] for r in range(world - 1))
        loads = [costs[c0:c1].sum() for c0, c1 in b]
        # contiguous slices: within one configuration of the ideal share
        assert max(loads) - costs.sum() / world <= costs.max()


def test_shard_bounds_edge_cases():
    assert shard_bounds([], 2) == [(0, 0), (0, 0)]
    assert shard_bounds([0, 0, 0], 2) == [(0, 2), (2, 3)]
    assert shard_bounds([5], 3) == [(0, 1), (1, 1), (1, 1)]
    with pytest.raises(ValueError):
        shard_bounds([1, 2], 0)


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, sizes, out_dir):
    import torch
    import torch.distributed as dist
    from oracle import debye_np as O
    from pyiid_gb300.distributed import (gather_rows, local_slice,
                                         max_over_ranks)
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        rng = np.random.default_rng(1)
        offsets = np.concatenate([[0], np.cumsum(sizes)])
        pos = rng.normal(0, 4, (offsets[-1], 3))
        species = np.zeros(offsets[-1], np.int32)
        c0, c1, loc, (a0, a1), sp = local_slice(offsets, species, rank, world)
        k = 40
        tab = np.ones((1, k), np.float32)
        rows = []
        for c in range(c1 - c0):
            p = pos[a0 + loc[c]:a0 + loc[c + 1]]
            rows.append(O.fq(p, np.repeat(tab, len(p), 0), 0.1))
        local = torch.as_tensor(np.array(rows).reshape(c1 - c0, k))
        from pyiid_gb300.distributed import shard_bounds, pair_costs
        full = gather_rows(local, shard_bounds(pair_costs(offsets), world))
        t = max_over_ranks(float(rank + 1))
        if rank == 0:
            np.save(os.path.join(out_dir, 'full.npy'), full.numpy())
            np.save(os.path.join(out_dir, 'tmax.npy'), np.array([t]))
    finally:
        dist.destroy_process_group()


def test_two_ranks_evaluate_their_slices_and_gather_in_order(tmp_path):
    import torch.multiprocessing as mp
    from oracle import debye_np as O
    sizes = [7, 3, 12, 5, 9, 2]
    port = _free_port()
    mp.spawn(_worker, args=(2, port, sizes, str(tmp_path)), nprocs=2,
             join=True)
    full = np.load(tmp_path / 'full.npy')
    rng = np.random.default_rng(1)
    offsets = np.concatenate([[0], np.cumsum(sizes)])
    pos = rng.normal(0, 4, (offsets[-1], 3))
    tab = np.ones((1, 40), np.float32)
    for c in range(len(sizes)):
        p = pos[offsets[c]:offsets[c + 1]]
        ref = O.fq(p, np.repeat(tab, len(p), 0), 0.1)
        assert np.array_equal(full[c], ref)
    assert np.load(tmp_path / 'tmax.npy')[0] == 2.0
