"""Benchmark: cell-updates/s of the swept KS solver (FP64) on GB300.

Workload (one "step"): the KS1D FP64 swept run of the benchmark table --
periodic, nx = 2^20, tpb = 256, dx = 0.5, dt = 0.005, tf = 200 (40000 time
steps), IC u(x,0) = 2 cos(19 pi x / 128) -- advanced from the IC to tf through
the C ABI (sw_run_device, state resident in HBM).  Between steps the state is
reset to the IC and L2 is flushed (a 256 MiB write); both are outside the
per-step CUDA-event timing.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

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
# FP64 operations per cell-update of the swept cell path: 2 sub-steps x 14 (exact power-of-two
# folds; each cell's square formed once and shared with both neighbours): 5 FMA, 4 MUL, 5 ADD.
DP_OPS_PER_UPDATE = 28
# FP64 pipe issue rates of this GB300 pool, measured with a throughput probe
# (152 SMs at 2.07 GHz): DFMA 0.627e12/s (1.99 per clock per SM, 1.25 TFLOP/s),
# DADD and DMUL 0.528e12/s.  The swept KS sub-step's mix (5 FMA, 9 MUL/ADD)
# issues at 14 / (5 / 0.627 + 9 / 0.528) = 0.560e12 operations/s.
FP64_OPS_PEAK = 0.627e12
FP64_KS_MIX_PEAK = 14.0 / (5.0 / 0.627e12 + 9.0 / 0.528e12)
METRIC = "cell-updates/s (KS1D FP64 swept, nx=2^20, tpb=256, dt=0.005, tf=200)"
WORKLOAD = ("KS1D FP64 swept (alg 1), periodic, nx=2^20, tpb=256, dx=0.5, dt=0.005, tf=200 "
            "(40000 time steps per step)")
K40_KS_F64_SWEPT_PUBLISHED = 1.07e10  # the reference's published KS FP64 swept figure, nx=2^20, on a K40c
# DRAM bytes (read + write) of one diamond launch of this workload from one ncu
# capture of this launch (cold-cache replay): 16.80 MB read + 0.84 MB written.
DIAMOND_TRAFFIC_BYTES = 17640000


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
    oracle.classic(c, u, 4, threads=threads)
    per_step = max((time.perf_counter() - t0) / 4, 1e-6)
    n = max(4, int(seconds / per_step))
    t0 = time.perf_counter()
    out = oracle.classic(c, u, n, threads=threads)
    dt = time.perf_counter() - t0
    assert np.isfinite(out).all()
    return {"value": NX * n / dt, "unit": "cell-updates/s", "cores": threads, "kind": "port",
            "sample": "classic KS FP64, nx=2^20, %d of the %d time steps (%.1f s), C/OpenMP oracle" % (n, NSTEPS, dt)}


def run_reference(args) -> None:
    world, rank, _ = _dist()
    if rank != 0:
        return
    seconds = max(2.0, 8.0 / max(1, args.steps + args.warmup) * 3)
    for _ in range(args.warmup):
        cpu_baseline(seconds=1.0)
    vals = []
    t_all = time.perf_counter()
    for _ in range(args.steps):
        vals.append(cpu_baseline(seconds=seconds))
    wall = time.perf_counter() - t_all
    v = statistics.median([x["value"] for x in vals])
    line = {
        "impl": "reference", "metric": METRIC,
        "value": v, "unit": "cell-updates/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": wall * 1e3 / max(1, args.steps), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic: reference KS IC 2cos(19 pi x/128)",
        "config": {"workload": WORKLOAD, "nx": NX, "tpb": TPB, "time_steps_per_step": NSTEPS,
                   "note": "the reference's programs need a GPU; this arm times the C/OpenMP port of its classic "
                           "scheme (the same cell-updates, bit for bit) on the host cores, on a bounded sample "
                           "of the time steps"},
        "cpu_baseline": {"value": v, "unit": "cell-updates/s", "cores": vals[0]["cores"], "kind": "port",
                         "sample": vals[0]["sample"]},
        "e2e": {"value": v, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


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
    stream = torch.cuda.current_stream()
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
        res = solver.run_device(c, state.data_ptr(), stream.cuda_stream)
        ev1.record(stream)
        ev1.synchronize()
        return ev0.elapsed_time(ev1), res

    for _ in range(args.warmup):
        one_step(cfg)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    times, launches, kern_ms, kern_launch = [], 0, 0.0, 0
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        for _ in range(args.steps):
            ms, res = one_step(cfg)
            times.append(ms)
            launches += res.launches
            kern_ms += res.kernel_ms
            kern_launch += res.launches
        torch.cuda.synchronize()
    clocks = clk.summary()
    value, total_ms = replica_throughput(sum(times), float(NX) * NSTEPS * args.steps)
    if world > 1:
        dist.barrier()
    ms_per_step = total_ms / args.steps

    final = state.cpu().numpy()
    assert np.isfinite(final).all()

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return

    # end to end through sw_run: host IC in, host final state out, copies inside the timing
    pinned_ic = torch.from_numpy(ic_host).pin_memory()
    e2e_ms = []
    for _ in range(max(1, min(args.steps, 2))):
        flush.fill_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fin, res, _ = solver.run(cfg, pinned_ic.numpy())
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_value = NX * NSTEPS / (statistics.median(e2e_ms) * 1e-3)

    # classic and variant on the same workload (the swept-vs-classic ratio), one run each
    extra = {}
    for name, alg in (("classic", sw.ALG_CLASSIC), ("variant", sw.ALG_VARIANT)):
        c2 = sw.make_config(sw.KS, 8, alg=alg, nx=NX, tpb=TPB, dt=DT, time_mode=sw.TIME_STEPS, n_steps=NSTEPS)
        ms, r2 = one_step(c2)
        extra[name] = {"value": NX * NSTEPS / (ms * 1e-3), "ms": ms, "launches": r2.launches}
    cfg32 = sw.make_config(sw.KS, 4, alg=sw.ALG_SWEPT, nx=NX, tpb=TPB, dt=DT, time_mode=sw.TIME_STEPS,
                           n_steps=NSTEPS)
    ic32 = torch.from_numpy(sw.initial_condition(cfg32)).cuda()
    st32 = ic32.clone()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    r32 = solver.run_device(cfg32, st32.data_ptr(), stream.cuda_stream)
    ev1.record(stream)
    ev1.synchronize()
    extra["fp32_swept"] = {"value": NX * NSTEPS / (ev0.elapsed_time(ev1) * 1e-3), "launches": r32.launches}

    hbm, peak_src = _peaks()
    launch_ms = kern_ms / max(1, kern_launch)
    steps_per_launch = TPB // 8
    alg_bytes = B_CLASSIC_KS_F64 * NX * steps_per_launch
    achieved = alg_bytes / (launch_ms * 1e-3) / 1e9
    roof = {"bound": "hbm", "kernel": "k_swept_group<KS,double,DIAMOND,4> (four 256-cell tiles per block)",
            "achieved": achieved, "peak": hbm,
            "unit": "GB/s", "frac": achieved / hbm, "peak_source": peak_src,
            "traffic": DIAMOND_TRAFFIC_BYTES, "traffic_source": "ncu dram__bytes_read+write, one diamond launch",
            "traffic_gbs": DIAMOND_TRAFFIC_BYTES / (launch_ms * 1e-3) / 1e9,
            "launch_ms": launch_ms,
            "algorithmic_bytes_per_launch": alg_bytes,
            "note": "effective bandwidth: classic KS FP64 bytes (40 B/cell-update) x cells x 32 steps per "
                    "diamond launch; the swept kernel's real DRAM traffic is far lower, its bound is the FP64 pipe"}
    dp = NX * steps_per_launch * DP_OPS_PER_UPDATE / (launch_ms * 1e-3)
    roof["fp64_pipe"] = {"achieved": dp / 1e12, "unit": "Tops/s", "ops_per_cell_update": DP_OPS_PER_UPDATE,
                         "peak": FP64_OPS_PEAK / 1e12, "frac": dp / FP64_OPS_PEAK,
                         "ks_mix_peak": FP64_KS_MIX_PEAK / 1e12, "frac_of_ks_mix": dp / FP64_KS_MIX_PEAK,
                         "peak_source": "measured (FP64 throughput probe on this GB300 pool)"}

    base = cpu_baseline(seconds=10.0) if world == 1 else None
    line = {
        "metric": METRIC,
        "value": value, "unit": "cell-updates/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": value / K40_KS_F64_SWEPT_PUBLISHED, "dtype": "f64",
        "data": "synthetic: the reference KS IC u(x,0) = 2cos(19 pi x/128)",
        "config": {"workload": WORKLOAD + ", state resident in HBM",
                   "nx": NX, "tpb": TPB, "time_steps_per_step": NSTEPS, "alg": "swept",
                   "l2": "flushed between steps (256 MiB write), outside the step timing",
                   "vs_baseline_source": "the reference's published KS FP64 swept figure, nx=2^20, K40c: 1.07e10 cell-updates/s"},
        "e2e": {"value": e2e_value, "unit": "cell-updates/s", "h2d_bytes_per_step": NX * 8,
                "d2h_bytes_per_step": NX * 8, "api": "sw_run (host IC -> host final state)"},
        "roofline": roof,
        "cpu_baseline": base,
        "clocks": clocks,
        "gpu_launches": launches,
        "classic": extra["classic"], "variant": extra["variant"], "fp32_swept": extra["fp32_swept"],
        "swept_over_classic": value / world / extra["classic"]["value"],
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
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
