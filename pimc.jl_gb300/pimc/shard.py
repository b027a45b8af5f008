"""Independent chains split across GPUs, one process per GPU.

The reference runs independent simulations side by side with
Distributed.pmap over parameter sets
(examples/density_2d_harmonically_trapped_bose_gas.jl:5,56).  Here a batch of
chains is split across ranks by longest-processing-time (LPT) order on the
same per-chain cost the engine uses to order its work queue (staging and
centre-of-mass work ~ N M, times 4 with the pair interaction; swaps ~ N^2/2),
each rank runs its shard as one engine batch on its own GPU, and the only
exchange is a host-side gather of the estimator sums at the end: chains never
talk to each other, so no device collective is involved.
"""
from __future__ import annotations

import heapq

import numpy as np


def chain_cost(p) -> float:
    """the engine's work-queue cost of one chain (ChainParams or a dict)"""
    get = (lambda k: p[k]) if isinstance(p, dict) else (lambda k: getattr(p, k))
    N, M = get("N"), get("M")
    inter = get("interactions")
    return float(N) * M * (4.0 if inter else 1.0) + 0.5 * float(N) * N


def lpt_partition(costs, nparts: int):
    """indices of the items split into nparts shards by LPT: items in
    decreasing cost, each to the currently lightest shard (ties to the lowest
    rank).  Returns (shards, loads); every index appears in exactly one
    shard, in increasing order within it."""
    if nparts < 1:
        raise ValueError("nparts must be >= 1")
    costs = np.asarray(costs, dtype=float)
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    heap = [(0.0, r) for r in range(nparts)]
    shards = [[] for _ in range(nparts)]
    loads = [0.0] * nparts
    for i in order:
        load, r = heapq.heappop(heap)
        shards[r].append(i)
        loads[r] = load + costs[i]
        heapq.heappush(heap, (loads[r], r))
    return [sorted(s) for s in shards], loads


def shard_of(params, rank: int, world: int):
    """this rank's chain indices of a batch (LPT on chain_cost)"""
    shards, _ = lpt_partition([chain_cost(p) for p in params], world)
    return shards[rank]


def gather_sums(pg, index, sums, counts, nchains: int):
    """the estimator sums of every chain of the batch, gathered from the
    ranks that ran them: index[k] is the global chain of local row k,
    sums[k][q] its running sums, counts[k] its measurements.  pg is
    torch.distributed (initialised) or None for one process.  Returns
    (sums[nchains][q], counts[nchains]) on every rank."""
    sums = np.asarray(sums, dtype=np.float64)
    q = sums.shape[1] if sums.ndim == 2 else 1
    full = np.zeros((nchains, q))
    cnt = np.zeros(nchains)
    full[np.asarray(index, dtype=int)] = sums.reshape(len(index), q)
    cnt[np.asarray(index, dtype=int)] = np.asarray(counts, dtype=np.float64)
    if pg is None:
        return full, cnt
    import torch
    t = torch.from_numpy(np.concatenate([full.ravel(), cnt]))
    if pg.get_backend() == "nccl":
        t = t.cuda()
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    t = t.cpu().numpy()
    return t[: nchains * q].reshape(nchains, q), t[nchains * q:]
