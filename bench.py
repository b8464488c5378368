"""Benchmark: cell-updates/s of the swept KS solver (FP64) on GB300, plus the
timed lines of every other target of the workload table.

Headline workload (one "step"): the KS1D FP64 swept run -- periodic,
nx = 2^20, tpb = 256, dx = 0.5, dt = 0.005, tf = 200 (40000 time steps), IC
u(x,0) = 2 cos(19 pi x / 128) -- advanced from the IC to tf through the C ABI
(sw_run_device, state resident in HBM).  Between steps the state is reset to
the IC and L2 is flushed (a 256 MiB write); both are outside the per-step
CUDA-event timing.  `e2e` is the same solve through sw_run with host buffers
(the IC's host-to-device and the final state's device-to-host copies inside
the timing).

`targets` (one GPU only): the other configurations, each timed on the device
by the library's own events and each checked bit for bit against our classic
scheme on the same run:
  * swept_over_classic_2e22 -- Heat, KS and Euler at nx = 2^22, FP64 and FP32,
    over a stated window of time steps, each swept run at its fastest measured
    tile width (perf.py's sweep);
  * cfg1 -- Heat FP64, periodic, nx = 4096, tpb = 128, Fourier number 0.1,
    20000 steps, with the error against the scheme's exact decaying mode;
  * cfg3 -- Euler/Sod FP64, nx = 2^22, tpb = 512, dt/dx = 0.1, a window of
    steps (t = 0.2 would take 8.4e6 steps);
  * cfg4 -- the 4096-domain KS ensemble (nx log-uniform in 2^10..2^16): FP32
    to tf = 100, FP64 over a window, tile chosen by the autotuner;
  * cfg5 -- the surrogate-corrected coarse KS ensemble (closure.bench_target).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--no-targets]

Prints one JSON line (rank 0).  N > 1 (torchrun): every rank solves its own
replica of the workload (the domains are independent; no collective on the
data path); value = N * cells * steps / max-over-ranks time.

--impl reference times the reference's classic scheme on the host cores: the
reference programs run only on a GPU, so the arm is the C/OpenMP restatement
of their classic schemes (oracle/, a port), on the same configuration, each
step a bounded sample of it.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

NX = 1 << 20
TPB = 256
DX = 0.5
DT = 0.005
TF = 200.0
NSTEPS = 40000            # tf / dt
B_CLASSIC_KS_F64 = 40     # algorithmic bytes per cell-update of the classic KS FP64 scheme
# FP64 operations per sub-step of the swept KS cell path (csrc/stencils.cuh ks_rhs_sq, after
# the exact power-of-two folding): 5 FMA, 2 general multiplies, 5 adds -- the work count of the
# roofline.  The exact products 6c and (l + r - 2c) * d2 are not counted (bit operations on the
# integer pipe); the 2 general multiplies (by dt and the new value's square) also run on the
# integer pipe (mul_int_fast), so the FP64 pipe itself issues 5 FMA and 5 adds per sub-step.
KS_SUBSTEP_MIX = {"fma": 5, "mul": 2, "add": 5}
KS_SUBSTEP_FP64_PIPE = {"fma": 5, "add": 5}
KS_OPS_PER_UPDATE = 2 * sum(KS_SUBSTEP_MIX.values())
KS_FP64_PIPE_OPS_PER_UPDATE = 2 * sum(KS_SUBSTEP_FP64_PIPE.values())
METRIC = "cell-updates/s (KS1D FP64 swept, nx=2^20, tpb=256, dt=0.005, tf=200)"
WORKLOAD = ("KS1D FP64 swept (alg 1), periodic, nx=2^20, tpb=256, dx=0.5, dt=0.005, tf=200 "
            "(40000 time steps per step)")
K40_KS_F64_SWEPT_PUBLISHED = 1.07e10  # the reference's published KS FP64 swept figure, nx=2^20, on a K40c
# DRAM bytes (read + write) of one diamond launch of this workload, from the ncu capture
# summarised in profiles/ks_f64_swept_diamond_nx2e20.md (cold-cache replay: 16.83 MB read,
# 0.06 MB written).
DIAMOND_TRAFFIC_BYTES = 16882176
DIAMOND_TRAFFIC_SOURCE = "profiles/ks_f64_swept_diamond_nx2e20.md (ncu dram__bytes_read.sum + dram__bytes_write.sum)"


def bench_config() -> dict:
    """The `config` both arms print (the same dict, so that the lines compare)."""
    return {"workload": WORKLOAD, "nx": NX, "tpb": TPB, "dx": DX, "dt": DT, "tf": TF,
            "time_steps_per_step": NSTEPS, "alg": "swept", "precision": "f64",
            "l2": "flushed between steps (256 MiB write), outside the step timing"}


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = Path("/tmp/sw_bench_clocks_%d.csv" % os.getpid())

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self) -> dict:
        if self.proc is None or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.path.read_text().splitlines():
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        self.path.unlink(missing_ok=True)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def replica_throughput(local_ms: float, units: float) -> tuple[float, float]:
    """Whole-job throughput of N independent replicas: every rank processed
    `units` cell-updates in `local_ms`; the job took the slowest rank's time.
    Returns (N * units / max_ms in units/s, max_ms).  Single process: no collective."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return units / (local_ms * 1e-3), local_ms
    world = dist.get_world_size()
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([local_ms], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    max_ms = float(t.item())
    return world * units / (max_ms * 1e-3), max_ms


def cpu_baseline(seconds: float = 10.0, threads: int | None = None) -> dict:
    """Oracle (C/OpenMP port of the reference classic KS) on the host cores, a
    bounded sample of the workload: nx = 2^20, as many classic steps as fill
    about `seconds`."""
    import numpy as np

    import oracle
    threads = threads or os.cpu_count() or 1
    c = oracle.reference_consts(oracle.KS, 8, NX, DT)
    u = oracle.reference_ic(oracle.KS, 8, NX)
    t0 = time.perf_counter()
    oracle.classic(c, u, 8, threads=threads)
    per_step = max((time.perf_counter() - t0) / 8, 1e-6)
    n = max(8, int(seconds / per_step))
    t0 = time.perf_counter()
    out = oracle.classic(c, u, n, threads=threads)
    dt = time.perf_counter() - t0
    assert np.isfinite(out).all()
    return {"value": NX * n / dt, "unit": "cell-updates/s", "cores": threads, "kind": "port",
            "sample": "classic KS FP64, nx=2^20, %d of the %d time steps (%.1f s), C/OpenMP oracle, %d threads"
                      % (n, NSTEPS, dt, threads)}


def run_reference(args) -> None:
    world, rank, _ = _dist()
    if rank != 0:
        return
    for _ in range(args.warmup):
        cpu_baseline(seconds=1.0)
    # each step a ~10 s sample, shortened only where many steps would take the
    # arm past four minutes
    per_step = min(10.0, max(4.0, 240.0 / max(1, args.steps)))
    vals = []
    t_all = time.perf_counter()
    for _ in range(args.steps):
        vals.append(cpu_baseline(seconds=per_step))
    wall = time.perf_counter() - t_all
    v = statistics.median([x["value"] for x in vals])
    line = {
        "impl": "reference", "metric": METRIC,
        "value": v, "unit": "cell-updates/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": wall * 1e3 / max(1, args.steps), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic: the reference KS IC u(x,0) = 2cos(19 pi x/128)",
        "config": bench_config(),
        "note": "the reference's programs need a GPU and its sources are not on this box; this arm times the "
                "C/OpenMP port of its classic scheme (the same cell-updates, bit for bit) on every host thread, "
                "each step a ~%.0f s sample of the time steps; value = the median step" % per_step,
        "cpu_baseline": {"value": v, "unit": "cell-updates/s", "cores": vals[0]["cores"], "kind": "port",
                         "sample": vals[0]["sample"]},
        "e2e": {"value": v, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------- targets
def _device_ic(sw, cfg, ic=None):
    """The IC in device layout (Euler: 4 values per cell) as a CUDA tensor."""
    import numpy as np
    import torch
    ic = sw.initial_condition(cfg) if ic is None else ic
    if cfg.problem == sw.EULER:
        dev = np.zeros((cfg.nx, 4), dtype=ic.dtype)
        dev[:, :3] = ic.reshape(-1, 3)
        ic = dev.ravel()
    return torch.from_numpy(np.ascontiguousarray(ic)).cuda()


def _time_run(sw, solver, cfg, ic_dev, warm_steps: int):
    """Warm the path on a short run, then run cfg from ic_dev; returns
    (cell-updates/s, kernel ms, launches, final device state)."""
    import ctypes as C
    import torch
    w = sw.Config()
    C.memmove(C.byref(w), C.byref(cfg), C.sizeof(sw.Config))
    w.n_steps = warm_steps
    solver.run_device(w, ic_dev.clone().data_ptr())
    st = ic_dev.clone()
    torch.cuda.synchronize()
    res = solver.run_device(cfg, st.data_ptr())
    return cfg.nx * cfg.n_steps / (res.kernel_ms * 1e-3), res.kernel_ms, res.launches, st


def _pair(sw, solver, problem, prec, nx, tpb, steps, dt, bc=0, ic=None, variant=False):
    """Classic and swept (and the variant) on one configuration: rates, times
    and bit-equality with classic."""
    import torch
    out = {"nx": nx, "tpb": tpb, "time_steps": steps, "dt": dt}
    cfgs = {"classic": sw.ALG_CLASSIC, "swept": sw.ALG_SWEPT}
    if variant:
        cfgs["variant"] = sw.ALG_VARIANT
    finals = {}
    for name, alg in cfgs.items():
        cfg = sw.make_config(problem, prec, alg=alg, nx=nx, tpb=tpb, dt=dt, bc=bc, time_mode=sw.TIME_STEPS,
                             n_steps=steps)
        ic_dev = _device_ic(sw, cfg, ic)
        rate, ms, launches, st = _time_run(sw, solver, cfg, ic_dev, warm_steps=min(steps, tpb))
        out[name] = {"cell_updates_per_s": rate, "kernel_ms": ms, "launches": launches}
        finals[name] = st
    out["swept_over_classic"] = out["swept"]["cell_updates_per_s"] / out["classic"]["cell_updates_per_s"]
    out["identical_to_classic"] = bool(torch.equal(finals["swept"], finals["classic"]))
    if variant:
        out["variant_identical_to_classic"] = bool(torch.equal(finals["variant"], finals["classic"]))
    out["finite"] = bool(torch.isfinite(finals["swept"]).all())
    return out, finals


def target_2e22(sw, solver) -> dict:
    big = 1 << 22
    rows = {}
    for key, problem, prec, tpb, steps, dt in (
            ("heat_f64", 0, 8, 1024, 4096, 0.004), ("heat_f32", 0, 4, 1024, 4096, 0.004),
            ("ks_f64", 1, 8, 128, 2048, DT), ("ks_f32", 1, 4, 1024, 2048, DT),
            ("euler_f64", 2, 8, 512, 512, 0.1 / (big - 2)), ("euler_f32", 2, 4, 512, 512, 0.1 / (big - 2))):
        rows[key], _ = _pair(sw, solver, problem, prec, big, tpb, steps, dt)
    return rows


def target_cfg1(sw, solver) -> dict:
    """Heat FP64, periodic, nx = 4096, tpb = 128, Fo = 0.1, 20000 steps, IC
    100 sin(2 pi x / L) + 50.  The scheme's exact solution is that mode
    decaying by g = 1 - 2 Fo (1 - cos(2 pi / nx)) per step."""
    import numpy as np
    nx, tpb, steps, alpha, dx = 4096, 128, 20000, 8.418e-5, 0.001
    dt = 0.1 * dx * dx / alpha
    x = np.arange(nx)
    ic = 100.0 * np.sin(2.0 * np.pi * x / nx) + 50.0
    out, finals = _pair(sw, solver, 0, 8, nx, tpb, steps, dt, bc=sw.BC_PERIODIC, ic=ic, variant=True)
    cfg = sw.make_config(0, 8, nx=nx, tpb=tpb, dt=dt, bc=sw.BC_PERIODIC)
    fo = sw.constants(cfg).fourier
    g = 1.0 - 2.0 * fo * (1.0 - np.cos(2.0 * np.pi / nx))
    exact = 50.0 + 100.0 * g ** steps * np.sin(2.0 * np.pi * x / nx)
    cont = 50.0 + 100.0 * np.exp(-alpha * (2.0 * np.pi / (nx * dx)) ** 2 * steps * dt) * np.sin(2.0 * np.pi * x / nx)
    got = finals["swept"].cpu().numpy()
    out.update({"fourier": fo, "max_abs_error_vs_exact_discrete_mode": float(np.abs(got - exact).max()),
                "max_abs_error_vs_continuous_solution": float(np.abs(got - cont).max())})
    return out


def target_cfg3(sw, solver, rows_2e22: dict | None) -> dict:
    """Euler/Sod FP64, nx = 2^22, tpb = 512, dt/dx = 0.1: a window of time
    steps (t = 0.2 would take 8.4e6 steps)."""
    big = 1 << 22
    r = rows_2e22["euler_f64"] if rows_2e22 else _pair(sw, solver, 2, 8, big, 512, 512, 0.1 / (big - 2))[0]
    out = dict(r)
    out["t_reached"] = r["time_steps"] * r["dt"]
    out["window_note"] = "512 of the 8.4e6 time steps to t = 0.2; rates are per cell-update"
    return out


def target_cfg4(sw, solver) -> dict:
    """The 4096-domain KS ensemble (nx = 2^e, e uniform on 10..16, seeded;
    dx = 0.5, dt = 0.005; the reference-law ICs).  FP32: swept and variant to
    tf = 100 (20000 steps), classic over a 2048-step window (and swept over
    the same window, bit-checked against it).  FP64: swept and classic over a
    1024-step window.  Tile and threads from the autotuner."""
    import numpy as np
    import torch
    ens = importlib.import_module("1dsweptcuda_gb300.ensemble")
    nx, u = ens.make_ensemble(n_domains=4096)
    cells = float(nx.sum())
    out = {"domains": 4096, "cells": int(cells)}

    def run(prec, alg, steps, tpb):
        cfg = sw.make_config(sw.KS, prec, alg=alg, tpb=tpb, dt=DT, time_mode=sw.TIME_STEPS, n_steps=steps)
        st = torch.from_numpy(u.astype(np.float64 if prec == 8 else np.float32)).cuda()
        torch.cuda.synchronize()
        res = solver.run_batch_device(cfg, nx, st.data_ptr())
        return cells * steps / (res.kernel_ms * 1e-3), res, st

    for prec, key, full, window in ((4, "fp32", 20000, 2048), (8, "fp64", None, 1024)):
        tune_cfg = sw.make_config(sw.KS, prec, alg=sw.ALG_SWEPT, tpb=0, dt=DT, time_mode=sw.TIME_STEPS,
                                  n_steps=window)
        t0 = time.perf_counter()
        tuned = solver.tune(tune_cfg, nx)
        row = {"tile": tuned.tile, "threads": tuned.threads, "tuning_s": time.perf_counter() - t0}
        run(prec, sw.ALG_SWEPT, 2 * tuned.tile, 0)          # graph capture and warm-up
        r_sw, res_sw, s_sw = run(prec, sw.ALG_SWEPT, window, 0)
        r_cl, res_cl, s_cl = run(prec, sw.ALG_CLASSIC, window, 256)
        row["window"] = {"time_steps": window, "swept": r_sw, "classic": r_cl, "swept_over_classic": r_sw / r_cl,
                         "identical_to_classic": bool(torch.equal(s_sw, s_cl))}
        if full:
            r_full, res_full, s_full = run(prec, sw.ALG_SWEPT, full, 0)
            run(prec, sw.ALG_VARIANT, 2 * tuned.tile, 0)
            r_var, res_var, s_var = run(prec, sw.ALG_VARIANT, full, 0)
            row["tf_100"] = {"time_steps": full, "swept": r_full, "swept_s": res_full.kernel_ms * 1e-3,
                             "variant": r_var, "variant_identical_to_swept": bool(torch.equal(s_full, s_var)),
                             "finite": bool(torch.isfinite(s_full).all())}
        out[key] = row
    return out


def targets(sw, solver) -> dict:
    out = {}
    t0 = time.perf_counter()
    out["swept_over_classic_2e22"] = target_2e22(sw, solver)
    out["cfg1_heat_periodic_4096"] = target_cfg1(sw, solver)
    out["cfg3_euler_sod_2e22"] = target_cfg3(sw, solver, out["swept_over_classic_2e22"])
    out["cfg4_ks_ensemble_4096"] = target_cfg4(sw, solver)
    closure = importlib.import_module("1dsweptcuda_gb300.closure")
    if hasattr(closure, "bench_target"):
        out["cfg5_closure"] = closure.bench_target(solver)
    out["seconds"] = time.perf_counter() - t0
    return out


# ------------------------------------------------------------------ ours
def diamond_launch_ms(sw, solver, state, n: int = 200) -> float:
    """Average device time of one diamond launch of the headline workload,
    timed with CUDA events on the stream the launches go to."""
    import torch
    cfg = sw.make_config(sw.KS, 8, alg=sw.ALG_SWEPT, nx=NX, tpb=TPB, dt=DT)
    st = state.clone()
    slots = torch.empty(2 * NX, dtype=torch.float64, device="cuda")
    stream, handle = torch.cuda.current_stream(), sw.native.torch_stream()
    solver.swept_pass(cfg, 0, 0, st.data_ptr(), slots.data_ptr(), handle)
    for k in range(4):
        solver.swept_pass(cfg, 1, 1 - (k & 1), st.data_ptr(), slots.data_ptr(), handle)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for k in range(n):
        solver.swept_pass(cfg, 1, 1 - (k & 1), st.data_ptr(), slots.data_ptr(), handle)
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / n


def run_ours(args) -> None:
    import numpy as np
    import torch

    world, rank, local = _dist()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    sw = importlib.import_module("1dsweptcuda_gb300")
    solver = sw.Solver(local)
    stream, handle = torch.cuda.current_stream(), sw.native.torch_stream()
    cfg = sw.make_config(sw.KS, 8, alg=sw.ALG_SWEPT, nx=NX, tpb=TPB, dt=DT, time_mode=sw.TIME_STEPS, n_steps=NSTEPS)
    ic_host = sw.initial_condition(cfg)
    ic = torch.from_numpy(ic_host).cuda()
    state = torch.empty_like(ic)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def one_step(c):
        state.copy_(ic)
        flush.fill_(1)
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        res = solver.run_device(c, state.data_ptr(), handle)
        ev1.record(stream)
        ev1.synchronize()
        return ev0.elapsed_time(ev1), res

    for _ in range(args.warmup):
        one_step(cfg)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    times, launches = [], 0
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        for _ in range(args.steps):
            ms, res = one_step(cfg)
            times.append(ms)
            launches += res.launches
        torch.cuda.synchronize()
    clocks = clk.summary()
    value, total_ms = replica_throughput(sum(times), float(NX) * NSTEPS * args.steps)
    if world > 1:
        dist.barrier()
    ms_per_step = total_ms / args.steps
    final = state.clone()

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return

    # the timed result against our classic scheme on the same 40000 steps
    c_cls = sw.make_config(sw.KS, 8, alg=sw.ALG_CLASSIC, nx=NX, tpb=TPB, dt=DT, time_mode=sw.TIME_STEPS,
                           n_steps=NSTEPS)
    cls_ms, cls_res = one_step(c_cls)
    classic = {"value": NX * NSTEPS / (cls_ms * 1e-3), "ms": cls_ms, "launches": cls_res.launches}
    identical = bool(torch.equal(state, final))
    state.copy_(final)

    # end to end through sw_run: host IC in, host final state out, copies inside the timing
    pinned_ic = torch.from_numpy(ic_host).pin_memory()
    e2e_ms = []
    for _ in range(3):
        flush.fill_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fin, res, _ = solver.run(cfg, pinned_ic.numpy())
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_value = NX * NSTEPS / (statistics.median(e2e_ms) * 1e-3)
    e2e_same = bool(np.array_equal(fin, final.cpu().numpy()))

    # the dominant kernel: one diamond launch (four 256-cell tiles per block), alone
    launch_ms = diamond_launch_ms(sw, solver, ic)
    rates = solver.fp64_rates()
    mix_peak = sum(KS_SUBSTEP_MIX.values()) / sum(n / rates[k] for k, n in KS_SUBSTEP_MIX.items())
    pipe_peak = sum(KS_SUBSTEP_FP64_PIPE.values()) / sum(n / rates[k] for k, n in KS_SUBSTEP_FP64_PIPE.items())
    steps_per_launch = TPB // 8
    updates = NX * steps_per_launch
    ops = updates * KS_OPS_PER_UPDATE / (launch_ms * 1e-3)
    pipe_ops = updates * KS_FP64_PIPE_OPS_PER_UPDATE / (launch_ms * 1e-3)
    hbm, peak_src = _peaks()
    alg_bytes = B_CLASSIC_KS_F64 * updates
    roof = {"bound": "fp64_pipe", "kernel": "k_swept_group<KS,double,DIAMOND,4> (four 256-cell tiles per block)",
            "achieved": ops / 1e12, "peak": mix_peak / 1e12, "unit": "Tops/s", "frac": ops / mix_peak,
            "peak_source": "measured live in this run (sw_fp64_rates) for the kernel's FP64 operation mix",
            "note": "achieved counts the scheme's 24 FP64 operations per cell-update; 4 of them (the "
                    "general products) run on the integer pipe with the same bits, so fp64_pipe.frac is the "
                    "FP64 pipe's own utilisation",
            "ops_per_cell_update": KS_OPS_PER_UPDATE, "ops_mix_per_substep": KS_SUBSTEP_MIX,
            "fp64_rates_per_s": rates, "frac_of_dfma_rate": ops / rates["fma"],
            "fp64_pipe": {"ops_per_cell_update": KS_FP64_PIPE_OPS_PER_UPDATE, "achieved": pipe_ops / 1e12,
                          "peak": pipe_peak / 1e12, "frac": pipe_ops / pipe_peak,
                          "integer_pipe_products_per_cell_update": KS_OPS_PER_UPDATE - KS_FP64_PIPE_OPS_PER_UPDATE,
                          "note": "the operations the FP64 pipe itself issues: the two general products of a "
                                  "sub-step (counted in the 24) run on the integer pipe with the same bits "
                                  "(mul_int_fast), as do its two exact ones (mul6, mul_pow2; not counted)"},
            "launch_ms": launch_ms, "cell_updates_per_launch": updates,
            "traffic": DIAMOND_TRAFFIC_BYTES, "traffic_source": DIAMOND_TRAFFIC_SOURCE,
            "hbm": {"effective_gbs": alg_bytes / (launch_ms * 1e-3) / 1e9, "peak_gbs": hbm,
                    "frac": alg_bytes / (launch_ms * 1e-3) / 1e9 / hbm, "peak_source": peak_src,
                    "algorithmic_bytes_per_launch": alg_bytes,
                    "raw_dram_gbs": DIAMOND_TRAFFIC_BYTES / (launch_ms * 1e-3) / 1e9,
                    "note": "classic KS FP64 bytes (40 B per cell-update) over the diamond launch time; the "
                            "swept kernel moves 80x fewer DRAM bytes and is bound by the FP64 and integer pipes"}}

    base = cpu_baseline(seconds=10.0) if world == 1 else None
    tg = targets(sw, solver) if (world == 1 and not args.no_targets) else None
    line = {
        "metric": METRIC,
        "value": value, "unit": "cell-updates/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": value / K40_KS_F64_SWEPT_PUBLISHED, "dtype": "f64",
        "data": "synthetic: the reference KS IC u(x,0) = 2cos(19 pi x/128)",
        "config": bench_config(),
        "vs_baseline_source": "the reference's published KS FP64 swept figure, nx=2^20, K40c: 1.07e10 cell-updates/s",
        "e2e": {"value": e2e_value, "unit": "cell-updates/s", "h2d_bytes_per_step": NX * 8,
                "d2h_bytes_per_step": NX * 8, "api": "sw_run (host IC -> host final state)",
                "identical_to_device_run": e2e_same},
        "roofline": roof,
        "cpu_baseline": base,
        "clocks": clocks,
        "gpu_launches": launches,
        "classic": classic, "identical_to_classic": identical,
        "swept_over_classic": value / world / classic["value"],
        "targets": tg,
    }
    print(json.dumps(line), flush=True)
    solver.close()
    if world > 1:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-targets", action="store_true", help="the headline line only")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
