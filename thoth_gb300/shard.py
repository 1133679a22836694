"""Path sharding across processes (one GPU per process) and result pooling.

Paths are independent, so N processes price disjoint Sobol index blocks of the
same book: rank k takes sobol_skip + sum(paths of ranks < k) and a balanced
share of the paths, exactly as the reference cluster splits a request between
slaves (pricer/src/modes/run_cluster.cpp:308-340). Results are pooled with the
cluster's rules: path-weighted mean, trust in quadrature
(run_cluster.cpp:413-445). The only exchange is one sum of 2 * (products + 1)
doubles, done on the host or with torch.distributed.all_reduce.
"""
import copy

import numpy as np


def shard_counts(paths, world):
    base, extra = divmod(int(paths), int(world))
    return [base + (1 if k < extra else 0) for k in range(world)]


def shard(book, rank, world):
    """A copy of ``book`` restricted to this rank's Sobol block."""
    counts = shard_counts(book.paths, world)
    b = copy.copy(book)
    b.sobol_skip = book.sobol_skip + sum(counts[:rank])
    b.paths = counts[rank]
    b.seed = book.seed + rank  # pseudo-random streams differ per rank (mcl_configuration seed = k)
    return b


def pool(results, counts):
    """Pool per-rank results (dicts with premium/trust arrays and book_premium/book_trust)."""
    total = float(sum(counts))
    w = np.array(counts, dtype=np.float64) / total
    prem = sum(wk * np.asarray(r["premium"]) for wk, r in zip(w, results))
    trust = np.sqrt(sum(wk * wk * np.asarray(r["trust"]) ** 2 for wk, r in zip(w, results)))
    bp = sum(wk * r["book_premium"] for wk, r in zip(w, results))
    bt = float(np.sqrt(sum(wk * wk * r["book_trust"] ** 2 for wk, r in zip(w, results))))
    return dict(premium=prem, trust=trust, book_premium=float(bp), book_trust=bt)


def allreduce_pool(result, count, group=None):
    """Pool across a torch.distributed group: every rank gets the pooled result."""
    import torch
    import torch.distributed as dist
    n = len(result["premium"])
    v = np.concatenate([[count], count * np.asarray(result["premium"]), (count * np.asarray(result["trust"])) ** 2,
                        [count * result["book_premium"], (count * result["book_trust"]) ** 2]])
    t = torch.tensor(v, dtype=torch.float64)
    dist.all_reduce(t, group=group)
    v = t.numpy()
    total = v[0]
    return dict(premium=v[1:1 + n] / total, trust=np.sqrt(v[1 + n:1 + 2 * n]) / total,
                book_premium=float(v[1 + 2 * n] / total), book_trust=float(np.sqrt(v[2 + 2 * n]) / total))
