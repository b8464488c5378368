"""bench.py --gpus N runs N independent replicas (the swept domains share no
data); the only collective is the max of the ranks' times.  Checked here with
two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    local_ms = 100.0 * (rank + 1)            # rank 1 is the slow one
    value, max_ms = bench.replica_throughput(local_ms, 1e9)
    q.put((rank, value, max_ms))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(world))
    for rank, value, max_ms in got:
        assert max_ms == 200.0
        assert abs(value - world * 1e9 / 0.2) < 1.0


def test_single_process_needs_no_collective():
    import bench
    assert not dist.is_initialized()
    value, ms = bench.replica_throughput(50.0, 1e6)
    assert ms == 50.0 and abs(value - 2e7) < 1e-6
