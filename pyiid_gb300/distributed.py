"""Configuration sharding across ranks (one process per GPU), and one large
configuration split across ranks (:func:`fq_grad_sharded`).

Batches of configurations are independent units: rank r evaluates a
contiguous slice of them and nothing crosses ranks on the data path.  The
slices balance the Debye work, which grows with the pair count
n (n - 1) / 2 of each configuration, not with the configuration count.
Results return to every rank in configuration order only when a caller
asks for them (:func:`gather_rows`); timings combine as the maximum over
ranks (:func:`max_over_ranks`).
"""
import numpy as np

__all__ = ['pair_costs', 'shard_bounds', 'local_slice', 'gather_rows',
           'max_over_ranks', 'fq_grad_sharded']


def pair_costs(offsets):
    """Pairs per configuration of a CSR batch (offsets [B + 1])."""
    n = np.diff(np.asarray(offsets, np.int64))
    return n * (n - 1) // 2


def shard_bounds(costs, world):
    """Split configurations 0..B-1 into ``world`` contiguous ranges of
    nearly equal total cost: [(c0, c1) per rank].  Boundaries sit where
    the cumulative cost crosses r / world of the total (the first such
    configuration goes to the earlier rank)."""
    costs = np.asarray(costs, np.float64)
    b = len(costs)
    if world < 1:
        raise ValueError('world must be >= 1')
    total = costs.sum()
    if total <= 0:
        edges = [round(r * b / world) for r in range(world + 1)]
    else:
        cum = np.concatenate([[0.0], np.cumsum(costs)])
        edges = [0]
        for r in range(1, world):
            target = total * r / world
            # smallest c with cum[c] >= target, never behind the last edge
            c = int(np.searchsorted(cum, target, side='left'))
            edges.append(min(max(c, edges[-1]), b))
        edges.append(b)
    return [(edges[r], edges[r + 1]) for r in range(world)]


def local_slice(offsets, species, rank, world):
    """This rank's configurations of a CSR batch:
    (c0, c1, local offsets, atom range (a0, a1), local species)."""
    offsets = np.asarray(offsets, np.int64)
    c0, c1 = shard_bounds(pair_costs(offsets), world)[rank]
    a0, a1 = int(offsets[c0]), int(offsets[c1])
    local = (offsets[c0:c1 + 1] - a0).astype(np.int32)
    return c0, c1, local, (a0, a1), np.asarray(species)[a0:a1]


def gather_rows(local, bounds, group=None):
    """All-gather per-configuration rows [c1 - c0, ...] of every rank into
    [B, ...] in configuration order (torch.distributed; rows are padded to
    the largest slice for the collective)."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    sizes = [c1 - c0 for c0, c1 in bounds]
    width = max(sizes) if sizes else 0
    pad = torch.zeros((width,) + tuple(local.shape[1:]), dtype=local.dtype,
                      device=local.device)
    pad[:local.shape[0]] = local
    parts = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(parts, pad, group=group)
    return torch.cat([p[:s] for p, s in zip(parts, sizes)])


def max_over_ranks(value, device=None, group=None):
    """The maximum of a per-rank float over all ranks (1 process: value)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def fq_grad_sharded(positions, species, scatter, qbin, k_begin=0, group=None,
                    gather_grad=False, part_fn=None, finish_fn=None):
    """F(Q) and its gradient of ONE configuration split across the ranks of
    ``group`` (one GPU each).  Rank r evaluates part r of the tile list in one
    pass (``pyiid_fq_grad_part``): the complete gradient rows of its atoms
    and the raw Debye sums of the pairs its tiles own.  The only exchange is
    an all-reduce of the K raw sums (float64), after which every rank forms
    F(Q) (``pyiid_fq_from_sums``).  Gradient rows stay on their owner unless
    ``gather_grad`` (an all-reduce of the zero-filled [N, 3, K] array).

    part_fn(positions, species, scatter, qbin, k_begin, part, n_parts) ->
    (sums, grad, rows) and finish_fn(species, scatter, k_begin, sums) -> fq
    default to the device calls; they are parameters so that the exchange
    can be exercised on CPU ranks.

    Returns (fq [K], grad [N, 3, K], rows bool [N] of this rank's atoms)."""
    import torch.distributed as dist
    if part_fn is None or finish_fn is None:
        from . import debye
        part_fn = part_fn or debye.fq_grad_part
        finish_fn = finish_fn or debye.fq_from_sums
    if dist.is_available() and dist.is_initialized():
        rank, world = dist.get_rank(group), dist.get_world_size(group)
    else:
        rank, world = 0, 1
    sums, grad, rows = part_fn(positions, species, scatter, qbin, k_begin,
                               rank, world)
    if world > 1:
        dist.all_reduce(sums, op=dist.ReduceOp.SUM, group=group)
        if gather_grad:
            dist.all_reduce(grad, op=dist.ReduceOp.SUM, group=group)
    return finish_fn(species, scatter, k_begin, sums), grad, rows
