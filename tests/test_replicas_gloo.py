"""Multi-rank path of bench.py on CPU: two gloo ranks as independent
replicas; the whole-job value is the steps of all ranks over the slowest
rank's time, with no collective on the data path."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    elapsed = [2.0, 3.0][rank]   # rank 1 is the slow replica
    v, t = bench.replica_throughput(torch, world, 100, elapsed, device="cpu")
    dist.barrier()
    q.put((rank, v, t))
    dist.destroy_process_group()


def test_two_replicas_aggregate_over_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, v, t in res:
        assert t == 3.0
        assert v == pytest.approx(200 / 3.0)
