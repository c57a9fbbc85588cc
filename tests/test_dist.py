"""Multi-rank path of bench.py on CPU: two gloo ranks run the replica
aggregation (max step time over ranks, whole-job throughput)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms_local = 10.0 if rank == 0 else 25.0  # rank 1 is the slow replica
    ms, gteps = bench.aggregate(ms_local, 1_000_000, 4, world, dist, "cpu")
    q.put((rank, ms, gteps))
    dist.destroy_process_group()


def test_replica_aggregation_two_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, gteps in res:
        assert ms == 25.0                                   # max over ranks
        assert abs(gteps - 2 * 1_000_000 * 4 / 0.025 / 1e9) < 1e-12
