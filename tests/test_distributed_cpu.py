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


def _sharded_worker(rank, world, port, out_dir):
    """fq_grad_sharded's exchange on CPU ranks, with oracle stand-ins for the
    device part (rank r owns atoms i = r mod world and the pairs (i, j < i))
    and the device finish."""
    import torch
    import torch.distributed as dist
    from oracle import debye_np as O
    from pyiid_gb300.distributed import fq_grad_sharded
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        rng = np.random.default_rng(5)
        pos = rng.normal(0, 4, (23, 3))
        tab = np.ones((1, 30), np.float32)
        sp = np.zeros(len(pos), np.int32)

        def part_fn(p, s, t, qbin, kb, part, n_parts):
            f = t[s].astype(np.float64)
            q = np.asarray(p, np.float32).astype(np.float64)
            Q = np.arange(t.shape[1]) * qbin
            sums = np.zeros(t.shape[1])
            rows = np.arange(len(q)) % n_parts == part
            for i in np.flatnonzero(rows):
                r = np.sqrt(((q[i] - q[:i]) ** 2).sum(1))[:, None]
                sums += (f[i] * f[:i] * np.sin(Q * r) / r).sum(0)
            sums[:kb] = 0.0
            grad = O.grad_fq(p, t[s], qbin)
            grad[~rows] = 0.0
            grad[:, :, :kb] = 0.0
            return (torch.as_tensor(sums), torch.as_tensor(grad), rows)

        def finish_fn(s, t, kb, sums):
            with np.errstate(all='ignore'):
                f = 2 * np.nan_to_num(sums.numpy() / O.normalization(t[s]))
            f[:kb] = 0.0
            return torch.as_tensor(f)

        fq, grad, rows = fq_grad_sharded(pos, sp, tab, 0.1, 2,
                                         gather_grad=True, part_fn=part_fn,
                                         finish_fn=finish_fn)
        np.save(os.path.join(out_dir, f'fq{rank}.npy'), fq.numpy())
        np.save(os.path.join(out_dir, f'grad{rank}.npy'), grad.numpy())
        np.save(os.path.join(out_dir, f'rows{rank}.npy'), rows)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize('world', [2, 3])
def test_two_ranks_split_one_configuration_and_exchange_the_sums(tmp_path,
                                                                 world):
    import torch.multiprocessing as mp
    from oracle import debye_np as O
    port = _free_port()
    mp.spawn(_sharded_worker, args=(world, port, str(tmp_path)),
             nprocs=world, join=True)
    rng = np.random.default_rng(5)
    pos = rng.normal(0, 4, (23, 3))
    tab = np.ones((1, 30), np.float32)
    want_f = O.fq(pos, np.repeat(tab, len(pos), 0), 0.1)
    want_f[:2] = 0.0
    want_g = O.grad_fq(pos, np.repeat(tab, len(pos), 0), 0.1)
    want_g[:, :, :2] = 0.0
    rows = [np.load(tmp_path / f'rows{r}.npy') for r in range(world)]
    assert np.array_equal(np.sum(rows, axis=0), np.ones(len(pos)))
    for r in range(world):
        f = np.load(tmp_path / f'fq{r}.npy')
        g = np.load(tmp_path / f'grad{r}.npy')
        assert np.allclose(f, want_f, rtol=1e-12, atol=1e-12)
        assert np.allclose(g, want_g, rtol=1e-12, atol=1e-12)
