"""Sharding a batch of subhaloes across GPUs (one process per GPU).

Subhaloes are independent units of the unbinding path: the only exchange is a
host-side gather of per-subhalo results, so no device collective is needed.
The batch is split by greedy longest-processing-time assignment on an
estimated cost n log n (tree walk work per pass), largest first, which every
rank computes identically from the sizes alone.

    plan = plan_shards(sizes, world_size)          # list of index arrays
    local = take(batch, plan[rank])                # this rank's sub-batch
    order, energy, results = unbinder.unbind_batch(local)
    merged = gather_results(plan, rank, world_size, (order, energy, results))

or all of it in one call: unbind_sharded(unbinder, batch, rank, world_size).
"""
from __future__ import annotations

import heapq

import numpy as np


def subhalo_cost(n: np.ndarray) -> np.ndarray:
    n = np.asarray(n, np.float64)
    return n * np.log2(np.maximum(n, 2.0))


def plan_shards(sizes, world_size: int):
    """Greedy LPT: subhaloes by decreasing cost, each to the least-loaded rank
    (ties to the lowest rank).  Returns world_size sorted index arrays."""
    sizes = np.asarray(sizes, np.int64)
    cost = subhalo_cost(sizes)
    order = np.argsort(-cost, kind="stable")
    heap = [(0.0, r) for r in range(world_size)]
    heapq.heapify(heap)
    parts = [[] for _ in range(world_size)]
    for s in order:
        load, r = heapq.heappop(heap)
        parts[r].append(int(s))
        heapq.heappush(heap, (load + float(cost[s]), r))
    return [np.array(sorted(p), np.int64) for p in parts]


def shard_loads(sizes, plan):
    cost = subhalo_cost(sizes)
    return np.array([cost[p].sum() for p in plan])


def take(batch: dict, idx: np.ndarray) -> dict:
    """The sub-batch of subhaloes idx (in that order), offsets rebuilt."""
    off = np.asarray(batch["offsets"], np.int64)
    spans = [np.arange(off[s], off[s + 1]) for s in idx]
    flat = np.concatenate(spans) if spans else np.zeros(0, np.int64)
    counts = np.array([off[s + 1] - off[s] for s in idx], np.int64)
    out = {"offsets": np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)}
    for k in ("id", "pos", "vel", "mass", "type"):
        out[k] = np.asarray(batch[k])[flat]
    for k in ("ref_pos", "ref_vel", "mostbound_pos", "mostbound_vel", "mostbound_id"):
        if k in batch:
            out[k] = np.asarray(batch[k])[idx]
    return out


def gather_results(plan, rank: int, world_size: int, local, group=None):
    """Gather every rank's (order, energy, results) to rank 0 (torch.distributed,
    any backend) and reassemble them in the batch's subhalo order.  Returns
    (order, energy, results) on rank 0 and None elsewhere."""
    import torch.distributed as dist
    objs = [None] * world_size if rank == 0 else None
    if world_size > 1:
        dist.gather_object(local, objs, dst=0, group=group)
    else:
        objs = [local]
    if rank != 0:
        return None
    nsub = sum(len(p) for p in plan)
    results = [None] * nsub
    orders = [None] * nsub
    energies = [None] * nsub
    for r, (order, energy, res) in enumerate(objs):
        pos = 0
        for k, s in enumerate(plan[r]):
            if "_n" not in res[k]:
                raise ValueError("each result must carry its subhalo's particle count '_n'")
            n = int(res[k]["_n"])
            orders[s] = order[pos:pos + n]
            energies[s] = energy[pos:pos + n]
            results[s] = res[k]
            pos += n
    return (np.concatenate(orders) if orders else np.zeros(0, np.int64),
            np.concatenate(energies) if energies else np.zeros(0, np.float32), results)


def unbind_sharded(unbinder, batch: dict, rank: int, world_size: int, group=None):
    """One batch unbound across world_size ranks: every rank plans the same
    split, unbinds its own shard with ``unbinder.unbind_batch`` (one call on its
    GPU, or any object with that method), and rank 0 gets the results of the
    whole batch in batch order, as one unbind_batch call of the whole batch
    would return them (None on the other ranks).  The only exchange is the
    host-side gather of the results."""
    sizes = np.diff(np.asarray(batch["offsets"], np.int64))
    plan = plan_shards(sizes, world_size)
    local = take(batch, plan[rank])
    order, energy, results = unbinder.unbind_batch(local)
    for k, s in enumerate(plan[rank]):
        results[k] = dict(results[k], _n=int(sizes[s]))
    out = gather_results(plan, rank, world_size, (order, energy, results), group=group)
    if out is None:
        return None
    order, energy, results = out
    for r in results:
        r.pop("_n", None)
    return order, energy, results
