"""Instance sharding of the batched runs (multigraph_gb300/shard.py) on CPU
ranks: two gloo processes split a source / seed list, each runs its share
through the oracle (standing in for its GPU), and the exchange must give
the unsplit oracle's answer on every rank -- BC scores summed, personalised
PageRank rows gathered in seed order."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from multigraph_gb300.shard import shard_bounds  # noqa: E402


def test_shard_bounds_cover_each_instance_once():
    for count in (0, 1, 5, 32, 256, 257):
        for world in (1, 2, 3, 8):
            seen = []
            sizes = []
            for r in range(world):
                lo, hi = shard_bounds(count, r, world)
                seen.extend(range(lo, hi))
                sizes.append(hi - lo)
            assert seen == list(range(count))
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_bounds(4, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


class _Graph:
    def __init__(self, nv):
        self.nv = nv


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    from multigraph_gb300.shard import bc_multi_sharded, ppr_batch_sharded
    from oracle import oracle as O
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        og = O.gen_rmat(10, 8, seed=5)
        g = _Graph(og.nv)
        src = np.random.default_rng(3).integers(0, og.nv, 21).astype(np.int32)
        bc = bc_multi_sharded(g, src, runner=lambda s: O.bc_multi_f64(og, s))
        seeds = src[:7]
        ppr = ppr_batch_sharded(g, seeds, runner=lambda s: np.stack(
            [O.ppr_f64(og, int(v), 0.85, 1e-10)[0].astype(np.float32) for v in s]))
        # a share can be empty: more ranks' worth of seeds than seeds
        one = ppr_batch_sharded(g, seeds[:1], runner=lambda s: np.stack(
            [O.ppr_f64(og, int(v), 0.85, 1e-10)[0].astype(np.float32) for v in s]))
        q.put((rank, bc, ppr, one))
    finally:
        dist.destroy_process_group()


def test_sharded_bc_and_ppr_two_ranks():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    from oracle import oracle as O
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=300) for _ in procs), key=lambda t: t[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    og = O.gen_rmat(10, 8, seed=5)
    src = np.random.default_rng(3).integers(0, og.nv, 21).astype(np.int32)
    ref = O.bc_multi_f64(og, src)
    rows = np.stack([O.ppr_f64(og, int(v), 0.85, 1e-10)[0].astype(np.float32) for v in src[:7]])
    for rank, bc, ppr, one in res:
        assert float(np.max(np.abs(bc - ref)) / np.max(np.abs(ref))) < 1e-12, rank
        assert np.array_equal(ppr, rows), rank
        assert np.array_equal(one, rows[:1]), rank
