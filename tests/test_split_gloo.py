"""A periodic domain split over ranks (1dsweptcuda_gb300/split.py): each rank
advances its contiguous part with swept passes as a periodic domain of its own,
and the ring exchange of the wrapping tile's slot (and, after a phase-1
down-triangle, its cells) makes the parts' concatenation equal the
single-domain run.  Run here on 1, 2 and 3 gloo ranks on the CPU, each pass
done by the NumPy model of the kernels' tile scheme (tests/swept_model.py),
and compared bit for bit with the oracle's classic scheme on the whole
domain."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _case(problem, prec, nx):
    import oracle
    if problem == 1:
        c = oracle.reference_consts(oracle.KS, prec, nx, 0.005)
        ic = oracle.reference_ic(oracle.KS, prec, nx)
    else:
        c = oracle.make_consts(oracle.HEAT, nx, prec=prec, bc=oracle.BC_PERIODIC, dt=0.004)
        x = np.arange(nx)
        ic = (50.0 + 100.0 * np.sin(2 * np.pi * x / nx)).astype(np.float64 if prec == 8 else np.float32)
    return c, ic


def _worker(rank, world, port, problem, prec, nx, W, n_steps, q):
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parent.parent
    sys.path[:0] = [str(root), str(root / "tests")]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import importlib
    split = importlib.import_module("1dsweptcuda_gb300.split")
    import swept_model
    c, ic = _case(problem, prec, nx)
    n = nx // world
    part = torch.from_numpy(ic[rank * n:(rank + 1) * n].copy())

    def pass_fn(mode, phase, state, slots):
        swept_model.swept_pass(problem, c, mode, phase, state.numpy(), slots.numpy(), W)

    passes = split.run_distributed(pass_fn, part, n_steps, problem, W)
    parts = [torch.empty_like(part) for _ in range(world)]
    dist.all_gather(parts, part)
    if rank == 0:
        q.put((torch.cat(parts).numpy(), passes))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world,problem,prec,nx,W,n_steps", [
    (2, 1, 8, 1024, 64, 56),    # KS FP64: 7 diamonds, the last down-triangle of phase 1 (cells move)
    (2, 1, 8, 1024, 64, 48),    # 6 diamonds: the down-triangle is phase 0 (no cells move)
    (3, 1, 4, 1536, 128, 64),   # three ranks in a ring, FP32
    (2, 0, 8, 512, 32, 48),     # Heat with periodic ends, 16 steps per diamond
    (1, 1, 8, 512, 64, 40),     # one rank: no exchange at all
])
def test_split_domain_equals_the_single_domain_run(world, problem, prec, nx, W, n_steps):
    import oracle
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, problem, prec, nx, W, n_steps, q))
             for r in range(world)]
    for p in procs:
        p.start()
    got, passes = q.get(timeout=300)
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    c, ic = _case(problem, prec, nx)
    want = oracle.classic(c, ic, n_steps)
    np.testing.assert_array_equal(got, want)
    q_steps = W // (2 * (1 if problem == 0 else 2) * (1 if problem == 0 else 2))
    assert passes == n_steps // q_steps + 1


def test_schedule_and_partition_rules():
    import importlib
    split = importlib.import_module("1dsweptcuda_gb300.split")
    assert split.schedule(24, 8) == [(0, 0), (1, 1), (1, 0), (2, 1)]
    assert split.schedule(16, 8) == [(0, 0), (1, 1), (2, 0)]
    with pytest.raises(ValueError):
        split.schedule(20, 8)          # not whole cycles
    assert split.check_partition(4096, 4, 256) == 1024
    with pytest.raises(ValueError):
        split.check_partition(4096, 3, 256)
    with pytest.raises(ValueError):
        split.check_partition(1024, 8, 256)   # parts smaller than a tile
    with pytest.raises(ValueError):
        split.steps_per_diamond(2, 256)       # Euler has fixed ends: not split
