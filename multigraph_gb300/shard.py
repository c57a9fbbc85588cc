"""Instance sharding of the batched runs over GPUs, one process per GPU.

Multi-source BC and personalised PageRank are batches of independent
instances (sources, one-hot seeds), so N processes -- one per GPU, each with
the graph uploaded to its own device -- split the instance list and exchange
results once at the end:

  bc_multi_sharded  rank r runs its contiguous share of the sources through
                    mg_bc_multi; the per-rank score vectors (n values) are
                    summed across ranks in FP64 (one all-reduce);
  ppr_batch_sharded rank r runs its share of the seeds through mg_ppr_batch;
                    the rows are gathered so every rank holds the full
                    nseeds x n result in seed order.

The exchange goes through torch.distributed (NCCL between GPUs, gloo on
CPU); no rank waits on another inside a kernel.  The reference runs one
source per process (main.cu:52-86); this layer has no counterpart there.

`runner` replaces the per-rank GPU call (same arguments, same result
shape), which lets the split and the exchange be exercised on CPU ranks
with the oracle doing the per-rank work.
"""
from __future__ import annotations

from typing import Callable, Optional, Sequence

import numpy as np


def shard_bounds(count: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous share [lo, hi) of `count` instances for `rank` of `world`:
    the first count % world ranks take one extra, so shares differ by at most
    one and their concatenation in rank order is the whole list."""
    if world < 1 or not 0 <= rank < world or count < 0:
        raise ValueError(f"bad shard request: count={count} rank={rank} world={world}")
    base, extra = divmod(count, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def _dist(group):
    import torch.distributed as dist
    if not dist.is_initialized():
        raise RuntimeError("torch.distributed is not initialised")
    return dist, dist.get_world_size(group), dist.get_rank(group)


def _device_for(dist, group):
    import torch
    if dist.get_backend(group) == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def bc_multi_sharded(graph, sources: Sequence[int], group=None,
                     runner: Optional[Callable[[np.ndarray], np.ndarray]] = None, **kw) -> np.ndarray:
    """Multi-source BC scores over all `sources`, each rank running its share.

    Every rank passes the same source list; every rank returns the summed
    scores (FP64).  An empty share contributes zeros."""
    import torch
    dist, world, rank = _dist(group)
    src = np.ascontiguousarray(sources, dtype=np.int32)
    lo, hi = shard_bounds(len(src), rank, world)
    n = graph.nv
    if hi > lo:
        part = runner(src[lo:hi]) if runner is not None else graph.bc_multi(src[lo:hi], **kw)[0]
        part = np.asarray(part, dtype=np.float64)
    else:
        part = np.zeros(n, np.float64)
    if part.shape != (n,):
        raise ValueError(f"per-rank scores have shape {part.shape}, expected ({n},)")
    t = torch.from_numpy(part).to(_device_for(dist, group))
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.cpu().numpy()


def ppr_batch_sharded(graph, seeds: Sequence[int], group=None,
                      runner: Optional[Callable[[np.ndarray], np.ndarray]] = None, **kw) -> np.ndarray:
    """Personalised PageRank rows for all `seeds` (nseeds x n, seed order),
    each rank computing its share; every rank returns the whole matrix."""
    import torch
    dist, world, rank = _dist(group)
    s = np.ascontiguousarray(seeds, dtype=np.int32)
    n = graph.nv
    lo, hi = shard_bounds(len(s), rank, world)
    if hi > lo:
        rows = runner(s[lo:hi]) if runner is not None else graph.ppr_batch(s[lo:hi], **kw)[0]
        rows = np.asarray(rows, dtype=np.float32)
    else:
        rows = np.zeros((0, n), np.float32)
    if rows.shape != (hi - lo, n):
        raise ValueError(f"per-rank rows have shape {rows.shape}, expected ({hi - lo}, {n})")
    dev = _device_for(dist, group)
    # all_gather needs equal shapes: pad every share to the largest one
    width = shard_bounds(len(s), 0, world)[1]
    buf = torch.zeros((width, n), dtype=torch.float32, device=dev)
    if hi > lo:
        buf[:hi - lo] = torch.from_numpy(rows).to(dev)
    parts = [torch.empty_like(buf) for _ in range(world)]
    dist.all_gather(parts, buf, group=group)
    out = np.empty((len(s), n), np.float32)
    for r in range(world):
        a, b = shard_bounds(len(s), r, world)
        out[a:b] = parts[r][:b - a].cpu().numpy()
    return out
