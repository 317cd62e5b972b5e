"""Multi-GPU runs of this path are replicas (one independent system per GPU, no data exchange);
bench.py takes the slowest rank's time and counts all ranks' interactions.  Checked here with
two gloo ranks on the CPU."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import sys
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    slow = bench.max_over_ranks(1.0 + rank, dist)  # rank 1 is the slow one
    bench.barrier(dist)
    q.put((rank, slow, bench.replica_throughput(world, 4, 100.0, slow)))
    dist.destroy_process_group()


def test_two_replicas_max_time_and_throughput():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    ps = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    out = sorted(q.get(timeout=10) for _ in range(2))
    for rank, slow, thr in out:
        assert slow == 2.0
        assert thr == pytest.approx(2 * 4 * 100.0 / 2.0)
