"""Path sharding across ranks: world_size 2 over gloo on CPU, each rank pricing
its disjoint Sobol block with the oracle, pooled with one all-reduce."""
import os
import socket

import numpy as np
import torch.multiprocessing as mp

import oracle
from thoth_gb300 import shard, workloads as W


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
    book = W.heston_grid(paths=3001, calendar=True, months=(1, 3), strikes=(90, 100, 110))
    mine = shard.shard(book, rank, world)
    r = oracle.price_book(mine)
    pooled = shard.allreduce_pool(r, mine.paths)
    q.put((rank, mine.sobol_skip, mine.paths, pooled))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_pool_equals_single_run():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = [q.get(timeout=300) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    got.sort()
    assert [(g[1], g[2]) for g in got] == [(0, 1501), (1501, 1500)]   # disjoint, covering blocks
    book = W.heston_grid(paths=3001, calendar=True, months=(1, 3), strikes=(90, 100, 110))
    full = oracle.price_book(book)
    for _, _, _, pooled in got:
        np.testing.assert_allclose(pooled["premium"], full["premium"], rtol=1e-12, atol=1e-12)
        # trust pooled in quadrature: the cluster's rule, close to the single-run standard error
        np.testing.assert_allclose(pooled["trust"], full["trust"], rtol=0.05)


def test_host_pool_matches_cluster_rule():
    book = W.gbm_call(paths=4000, greeks=False)
    counts = shard.shard_counts(book.paths, 3)
    parts = [oracle.price_book(shard.shard(book, k, 3)) for k in range(3)]
    pooled = shard.pool(parts, counts)
    full = oracle.price_book(book)
    np.testing.assert_allclose(pooled["premium"], full["premium"], rtol=1e-12)
