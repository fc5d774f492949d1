"""Multi-GPU runs are independent replicas: the benchmark's whole-job value is
every rank's points over the slowest rank's time. The rank logic is checked
here with two gloo processes on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    local_ms = [120.0, 150.0][rank]
    value, t_max = bench.replica_throughput(local_ms, 1000, 3, world,
                                            bench.make_reduce_max(dist, torch, "cpu"))
    q.put((rank, value, t_max))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for _, value, t_max in res:
        assert t_max == 150.0
        assert abs(value - 1000 * 2 * 3 / 0.150) < 1e-6


def test_single_rank_needs_no_collective():
    import bench
    value, t = bench.replica_throughput(200.0, 10, 2, 1)
    assert t == 200.0 and abs(value - 100.0) < 1e-9
