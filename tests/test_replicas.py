"""Multi-GPU form of the channelizer is replicas only: each rank processes
its own stream with no exchange on the data path, and the job's numbers are
the slowest rank's time and the sum of all ranks' outputs.  The aggregation
bench.py uses is checked here with two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t, u = bench.replica_aggregate(10.0 + 5 * rank, 1000 * (rank + 1), world, torch.device("cpu"))
    q.put((rank, t, u))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_aggregate_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for _, t, u in res:
        assert t == 15.0          # the slowest rank's time
        assert u == 3000.0        # all ranks' outputs


def test_replica_aggregate_single_rank_is_identity():
    import bench
    assert bench.replica_aggregate(3.5, 7, 1, None) == (3.5, 7.0)
