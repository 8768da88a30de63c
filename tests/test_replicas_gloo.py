"""Multi-GPU form of the path: independent replicas (the reference has no distribution; one
instance per GPU, no data-path collective).  The host logic -- max-over-ranks job time and
whole-job throughput -- runs here as world_size-2 gloo ranks on the CPU."""
import os
import socket
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    local_ms = [100.0, 250.0][rank]                 # rank 1 is the slow one
    val, t_max = bench.replica_throughput(local_ms, cells=1_000_000, steps=10, dist=dist)
    q.put((rank, val, t_max))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_throughput_uses_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(2))
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, val, t_max in out:
        assert t_max == 250.0
        assert val == pytest.approx(2 * 1_000_000 * 10 / 0.25 / 1e9)


def test_single_process_throughput():
    sys.path.insert(0, ROOT)
    import bench
    val, t = bench.replica_throughput(50.0, cells=2_000_000, steps=5)
    assert t == 50.0 and val == pytest.approx(2e6 * 5 / 0.05 / 1e9)
