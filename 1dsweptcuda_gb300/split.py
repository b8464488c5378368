"""One periodic domain split into contiguous parts, each advanced by the swept
passes of its own device or process, with the edge exchange between
neighbouring parts (the multi-domain run of the reference's MPI comparison,
ResultPlots/ConferencePaper/KS_MPI.csv; the reference's MPI code itself is not
in its repository).

Partition.  A periodic KS or Heat domain of nx cells, tile width W, is cut into
P parts of n = nx / P cells (n a multiple of W); part r holds global cells
[r n, (r + 1) n) and 2 n cells of half-tile slots.  Each part runs
sw_swept_pass on its cells as if they were a periodic domain of n cells.
Every tile of the up-triangle and of a phase-0 pass lies inside its part.  In
a phase-1 pass the part's last tile wraps from its cell n - 1 to its cell 0;
in the domain that tile straddles parts r and r + 1 and must use part r + 1's
first slot.  Only that tile touches slot 0 in a phase-1 pass, so:

  * before a phase-1 pass, slot 0 moves one part to the left (part r receives
    part r + 1's slot 0, which its wrapping tile then reads);
  * after a phase-1 diamond, slot 0 moves back one part to the right (the
    wrapping tile's output for part r + 1's first half-tile);
  * after a phase-1 down-triangle, state cells [0, W/2) move one part to the
    right (the wrapping tile wrote part r + 1's first half-tile there).

Each exchange is W cells of slot (or W/2 of state) per part and neighbour,
point to point; nothing is reduced.  The arithmetic is the kernels' own, so the
parts' concatenated state equals the single-domain run bit for bit.  The
periodic boundary is what lets every part treat itself as periodic: the
stencils never look at a cell's global position (KS; Heat with periodic ends).

Runs cover whole swept cycles (n_steps a multiple of W / (2 R S) time steps):
a classic remainder step would need halo cells the parts do not exchange.

Two drivers share the schedule:
  * run_local: all parts on one device of this process; the exchanges are
    device-to-device copies (the single-GPU form, and the check of the
    exchange against the single-domain run);
  * run_distributed: one part per torch.distributed rank.  With NCCL the slots
    go point to point between GPUs; with another backend (gloo) device tensors
    are staged through host memory.  The pass itself is a callable, so the
    same exchange runs over any pass implementation.
"""
from __future__ import annotations

from typing import Callable, Sequence

UP, DIAMOND, DOWN = 0, 1, 2
RADIUS = {0: 1, 1: 2}     # Heat, KS
SUBSTEPS = {0: 1, 1: 2}


def steps_per_diamond(problem: int, tile: int) -> int:
    if problem not in RADIUS:
        raise ValueError("a split domain must be periodic: Heat (periodic ends) or KS")
    return tile // (2 * RADIUS[problem] * SUBSTEPS[problem])


def schedule(n_steps: int, q: int) -> list[tuple[int, int]]:
    """(mode, phase) of every pass of a swept run of n_steps time steps, q
    per diamond: the up-triangle, diamonds of phases 1, 0, 1, ..., and the
    down-triangle, for a whole number of diamonds."""
    if n_steps < q or n_steps % q:
        raise ValueError("a split run covers whole swept cycles: n_steps must be a positive multiple of %d" % q)
    full = n_steps // q
    return [(UP, 0)] + [(DIAMOND, d & 1) for d in range(1, full)] + [(DOWN, full & 1)]


def check_partition(nx: int, parts: int, tile: int) -> int:
    """Cells per part; raises unless nx splits into `parts` runs of whole tiles."""
    if parts < 1 or nx % parts or (nx // parts) % tile or nx // parts < tile:
        raise ValueError("nx = %d does not split into %d parts of whole %d-cell tiles" % (nx, parts, tile))
    return nx // parts


def part_config(sw, cfg, parts: int):
    """The configuration each part runs: the domain's, with nx = nx / parts."""
    import ctypes as C
    if cfg.problem == sw.EULER or (cfg.problem == sw.HEAT and cfg.bc != sw.BC_PERIODIC):
        raise ValueError("a split domain must be periodic: Heat (periodic ends) or KS")
    c = sw.Config()
    C.memmove(C.byref(c), C.byref(cfg), C.sizeof(sw.Config))
    c.nx = check_partition(int(cfg.nx), parts, int(cfg.tpb))
    return c


def run_local(solver, cfg, states: Sequence, n_steps: int) -> int:
    """Advance the parts `states` (CUDA tensors of nx / P cells each, in domain
    order) of one periodic domain by n_steps time steps on this process's
    device, passes and exchange copies in order on torch's current stream.
    cfg describes the whole domain (nx = P parts' cells).  Returns the passes
    launched per part."""
    import torch
    sw = _sw()
    stream = sw.native.torch_stream()
    P = len(states)
    pc = part_config(sw, cfg, P)
    W, h = int(cfg.tpb), int(cfg.tpb) // 2
    slots = [torch.empty(2 * s.numel(), dtype=s.dtype, device=s.device) for s in states]
    plan = schedule(n_steps, steps_per_diamond(cfg.problem, W))

    def shift(views, by):  # views[r] <- old views[(r + by) % P]
        old = [v.clone() for v in views]
        for r in range(P):
            views[r].copy_(old[(r + by) % P])

    for mode, phase in plan:
        if phase == 1 and P > 1:
            shift([sl[:W] for sl in slots], 1)
        for st, sl in zip(states, slots):
            solver.swept_pass(pc, mode, phase, st.data_ptr(), sl.data_ptr(), stream)
        if phase == 1 and P > 1:
            shift([sl[:W] for sl in slots] if mode == DIAMOND else [st[:h] for st in states], -1)
    return len(plan)


def run_distributed(pass_fn: Callable, state, n_steps: int, problem: int, tile: int, group=None) -> int:
    """Advance this rank's part `state` (a tensor of the part's cells) of one
    periodic domain split over the ranks of `group` (rank r holds part r) by
    n_steps time steps.  pass_fn(mode, phase, state, slots) runs one swept
    pass on the part (slots: a tensor of 2 * len(state) cells, kept here).
    Exchanges go to the ring neighbours only.  Returns the passes run."""
    import torch
    import torch.distributed as dist
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    W, h = tile, tile // 2
    if state.numel() % W:
        raise ValueError("a part must hold whole %d-cell tiles" % W)
    slots = torch.empty(2 * state.numel(), dtype=state.dtype, device=state.device)
    plan = schedule(n_steps, steps_per_diamond(problem, W))
    left, right = (rank - 1) % world, (rank + 1) % world
    if group is not None:
        left, right = dist.get_global_rank(group, left), dist.get_global_rank(group, right)
    staged = state.is_cuda and dist.get_backend(group) != "nccl"

    def exchange(view, to, frm):
        """view <- the neighbour `frm`'s view, while ours goes to `to`."""
        out = view.cpu() if staged else view.clone()
        buf = torch.empty_like(out)
        reqs = [dist.isend(out, to, group=group), dist.irecv(buf, frm, group=group)]
        for q in reqs:
            q.wait()
        view.copy_(buf)

    for mode, phase in plan:
        if phase == 1 and world > 1:
            exchange(slots[:W], left, right)
        pass_fn(mode, phase, state, slots)
        if phase == 1 and world > 1:
            exchange(slots[:W] if mode == DIAMOND else state[:h], right, left)
    return len(plan)


def _sw():
    import importlib
    return importlib.import_module("1dsweptcuda_gb300")
