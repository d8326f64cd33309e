"""Instance sharding of the batched cavities: a deterministic cost-balanced
partition, and the gather of per-instance results over two gloo ranks on CPU."""
import os
import socket

import numpy as np
import pytest

from plugin_navierstokes_gb300.sharding import shard_instances


def test_partition_covers_and_balances():
    from plugin_navierstokes_gb300 import mesh

    N, _, _ = mesh.draw_cavity_params(256, seed=3)
    cost = (N + 1.0) ** 2
    for world in (1, 2, 4, 8):
        parts = shard_instances(cost, world)
        allidx = np.concatenate(parts)
        assert np.array_equal(np.sort(allidx), np.arange(256))
        loads = [cost[p].sum() for p in parts]
        assert max(loads) - min(loads) <= cost.max()
    assert all(np.array_equal(a, b) for a, b in zip(shard_instances(cost, 4), shard_instances(cost, 4)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist

    from plugin_navierstokes_gb300.sharding import gather_results, shard_instances

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    cost = np.array([5, 1, 9, 3, 3, 7, 2], dtype=float)
    mine = shard_instances(cost, world)[rank]
    res = [{"instance": int(i), "rank": rank} for i in mine]
    allres = gather_results(res, mine, cost.size)
    dist.destroy_process_group()
    q.put((rank, [r["instance"] for r in allres], [r["rank"] for r in allres]))


def test_gather_over_two_gloo_ranks():
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = [q.get(timeout=120) for _ in ps]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, inst, owners in out:
        assert inst == list(range(7))
        assert set(owners) == {0, 1}
    assert out[0][1:] == out[1][1:]
