"""The N > 1 path of bench.py on CPU: replicas over a world-size-2 gloo
process group (no GPU).  Each rank times its own replica; the reported
duration is the maximum over ranks and the rate counts every rank's work
(weak scaling, no data-path collective)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms, value = bench.aggregate_over_ranks(100.0 * (rank + 1), 1_000_000, 4, dist)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, ms, value))


def test_replicas_take_the_max_time_and_sum_the_work():
    pytest.importorskip("torch")
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, value in out:
        assert ms == 200.0
        assert abs(value - 2 * 1_000_000 * 4 / 0.2 / 1e6) < 1e-9


def test_single_process_is_the_plain_rate():
    sys.path.insert(0, ROOT)
    import bench
    ms, value = bench.aggregate_over_ranks(50.0, 2_000_000, 5)
    assert ms == 50.0 and abs(value - 200.0) < 1e-9
