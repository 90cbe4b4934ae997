"""Multi-GPU sharding of a batch (hbtplus_gb300.shard), on CPU with gloo.

Two host processes (world size 2, gloo, 127.0.0.1) split the 2000-subhalo
batch with the planner, each produces per-subhalo results for its shard (a
stand-in for the GPU call: no GPU here), and rank 0 reassembles them in batch
order.  Checks: every subhalo is processed exactly once, the reassembled
order/energy arrays line up with the batch offsets, and the LPT loads are
balanced."""
import os
import socket

import numpy as np
import pytest

from hbtplus_gb300 import shard
from hbtplus_gb300 import synthetic as S


def fake_unbind(batch):
    """Deterministic per-subhalo results standing in for the GPU call."""
    off = batch["offsets"]
    order, energy, res = [], [], []
    for s in range(len(off) - 1):
        n = int(off[s + 1] - off[s])
        order.append(np.arange(n)[::-1])
        energy.append(batch["id"][off[s]:off[s + 1]].astype(np.float32))
        res.append({"nbound": n // 2, "_n": n, "first_id": int(batch["id"][off[s]]) if n else -1})
    return (np.concatenate(order) if order else np.zeros(0, np.int64),
            np.concatenate(energy) if energy else np.zeros(0, np.float32), res)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    b = S.subhalo_batch(nsub=300, seed=11, nmax=20000)
    sizes = np.diff(b["offsets"])
    plan = shard.plan_shards(sizes, world)
    local = shard.take(b, plan[rank])
    out = shard.gather_results(plan, rank, world, fake_unbind(local))
    if rank == 0:
        order, energy, res = out
        ok = len(res) == len(sizes)
        off = b["offsets"]
        for s in range(len(sizes)):
            n = int(sizes[s])
            ok &= res[s]["_n"] == n
            ok &= res[s]["first_id"] == (int(b["id"][off[s]]) if n else -1)
            ok &= np.array_equal(order[off[s]:off[s + 1]], np.arange(n)[::-1])
            ok &= np.array_equal(energy[off[s]:off[s + 1]], b["id"][off[s]:off[s + 1]].astype(np.float32))
        loads = shard.shard_loads(sizes, plan)
        q.put((bool(ok), float(loads.max() / loads.mean())))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gloo_shard_and_gather():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    ok, imbalance = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert ok
    assert imbalance < 1.05


def _oracle_worker(rank, world, port, q):
    """Each rank unbinds its shard with the C oracle (the stand-in for its
    GPU); rank 0 compares the gathered batch with one oracle call on the whole
    batch."""
    import torch.distributed as dist
    from helpers import OracleUnbinder
    from oracle import Oracle
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    b = S.subhalo_batch(nsub=60, seed=12, nmax=3000)
    p = S.default_params()
    un = OracleUnbinder(Oracle(), p)
    out = shard.unbind_sharded(un, b, rank, world)
    if rank == 0:
        order, energy, res = out
        o1, e1, r1 = un.unbind_batch(b)
        ok = np.array_equal(order, o1) and np.array_equal(energy, e1, equal_nan=True)
        ok &= len(res) == len(r1)
        for x, y in zip(res, r1):
            for k in y:
                ok &= np.array_equal(np.asarray(x[k]), np.asarray(y[k]), equal_nan=True)
        q.put(bool(ok))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_sharded_unbinding_equals_one_rank():
    """unbind_sharded over two gloo ranks gives, on rank 0, bit for bit the
    results of unbinding the whole batch in one place."""
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_oracle_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    ok = q.get(timeout=300)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert ok


def test_plan_is_a_partition_and_balanced():
    rng = np.random.Generator(np.random.PCG64(3))
    sizes = S.batch_sizes(rng, 2000)
    for world in (1, 2, 4, 8):
        plan = shard.plan_shards(sizes, world)
        allidx = np.sort(np.concatenate(plan))
        assert np.array_equal(allidx, np.arange(len(sizes)))
        loads = shard.shard_loads(sizes, plan)
        # LPT bound: max load <= mean + the largest single cost
        assert loads.max() <= loads.mean() + shard.subhalo_cost(sizes).max() + 1e-6
