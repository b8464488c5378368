"""Performance sweep (the role of the reference's quickperform.py / runTest.sh):
time classic, swept and variant over problems, precisions, nx and tpb with the
state resident on the device, and check that all paths agree bit for bit.

    python 1dsweptcuda_gb300/perf.py [--quick] [--ensemble] [--only TEXT] [--precision 4|8]
                                     [--threads 0,64,...] [--tpb 256,...] [--algs swept,...] [--json out.json]
    python 1dsweptcuda_gb300/perf.py --divide [Divides.txt]     # the KS division study alone

Each case runs SW_TIME_STEPS with a step count that is a whole number of swept
cycles for every tpb in the case, timed with CUDA events inside the library
(sw_result.kernel_ms).  Prints one row per case and the swept/classic ratio.
--threads times swept and variant at each listed threads per block (0 = the
library's default for the tile width).
"""
from __future__ import annotations

import argparse
import importlib
import json
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def cases(quick: bool):
    # (label, problem, precision, bc, nx, [tpb...], steps, dt)
    big = 1 << 22
    c = [
        ("heat-periodic nx=4096 (Fo=0.1)", 0, 8, 2, 4096, [128], 20480, 1.18793e-3),
        ("ks nx=2^20", 1, 8, 0, 1 << 20, [256], 4096, 0.005),
        ("heat nx=2^22", 0, 8, 0, big, [256, 1024], 4096, 0.004),
        ("heat nx=2^22", 0, 4, 0, big, [256, 1024], 4096, 0.004),
        ("ks nx=2^22", 1, 8, 0, big, [256, 1024], 2048, 0.005),
        ("ks nx=2^22", 1, 4, 0, big, [256, 1024], 2048, 0.005),
        ("euler nx=2^22", 2, 8, 0, big, [256, 512], 256, 0.1 / (big - 2)),
        ("euler nx=2^22", 2, 4, 0, big, [256, 512], 256, 0.1 / (big - 2)),
    ]
    if quick:
        c = [x for x in c if x[4] <= (1 << 20)]
    return c


def ensemble_rows(sw, solver, quick: bool):
    """Config 4 shape: 4096 periodic KS domains, nx log-uniform in 2^10..2^16 (seeded),
    dx = 0.5, dt = 0.005; swept (autotuned tile), variant and classic, FP32 and FP64,
    over a window of time steps (FP32: the full tf = 100, 20000 steps)."""
    import numpy as np
    import torch
    ens = __import__("importlib").import_module("1dsweptcuda_gb300.ensemble")
    nx, u = ens.make_ensemble(n_domains=256 if quick else 4096)
    rows = []
    for prec, steps in ((4, 1024 if quick else 20000), (8, 512 if quick else 2048)):
        dt = np.float64 if prec == 8 else np.float32
        ic = u.astype(dt)
        tuned = None
        out = {}
        for alg in (sw.ALG_SWEPT, sw.ALG_VARIANT, sw.ALG_CLASSIC):
            n = steps if alg != sw.ALG_CLASSIC else min(steps, 512)
            cfg = sw.make_config(sw.KS, prec, alg=alg, tpb=0 if alg != sw.ALG_CLASSIC else 256, dt=0.005,
                                 time_mode=sw.TIME_STEPS, n_steps=n)
            if alg == sw.ALG_SWEPT:
                tuned = solver.tune(cfg, nx)
            st = torch.from_numpy(ic.copy()).cuda()
            res = solver.run_batch_device(cfg, nx, st.data_ptr())
            ups = float(nx.sum()) * n / (res.kernel_ms * 1e-3)
            out[alg] = (st.cpu().numpy(), n)
            rows.append({"case": "ks ensemble 4096 domains" if not quick else "ks ensemble 256 domains",
                         "precision": prec, "alg": {1: "swept", 2: "variant", 0: "classic"}[alg],
                         "tile": res.tile, "threads": tuned.threads if tuned and alg else None,
                         "cells": int(nx.sum()), "steps": n, "ms": res.kernel_ms, "cell_updates_per_s": ups,
                         "launches": res.launches})
            print("%-34s f%-2d %-8s tile=%-5s %10.3e cell-updates/s (%d steps, %.1f ms)" % (
                rows[-1]["case"], prec * 8, rows[-1]["alg"], res.tile, ups, n, res.kernel_ms), flush=True)
        rows[-3]["equal_to_variant"] = bool(np.array_equal(out[1][0], out[2][0]))
        rows[-3]["tuning"] = tuned.candidates()
    return rows


def divide_rows(sw, solver, quick: bool, path: str | None):
    """The reference's division study (its Divides.txt: KS time per step with the
    DIVISE build against the reciprocal build, FP64 and FP32, nx = 2^11..2^20):
    KS swept, tpb = 256, dx = 0.5, dt = 0.005, SW_FLAG_KS_DIVIDE on and off.  At
    dx = 0.5 both forms must give the same bits.  Writes the table in the study's
    column order (nx, us/step divide FP64, multiply FP64, divide FP32, multiply
    FP32) when a path is given."""
    import numpy as np
    import torch
    stream = torch.cuda.current_stream()
    rows, table = [], []
    for e in range(11, 17 if quick else 21):
        nx = 1 << e
        steps = 4096
        line = [nx]
        for prec in (8, 4):
            outs = []
            for flags in (sw.FLAG_KS_DIVIDE, 0):
                cfg = sw.make_config(sw.KS, prec, alg=sw.ALG_SWEPT, nx=nx, tpb=256, dt=0.005, flags=flags,
                                     time_mode=sw.TIME_STEPS, n_steps=steps)
                ic = sw.initial_condition(cfg)
                st = torch.from_numpy(ic).cuda()
                solver.run_device(cfg, st.data_ptr(), stream.cuda_stream)  # warm
                st = torch.from_numpy(ic).cuda()
                torch.cuda.synchronize()
                res = solver.run_device(cfg, st.data_ptr(), stream.cuda_stream)
                outs.append(st.cpu().numpy())
                us = res.kernel_ms * 1e3 / steps
                line.append(us)
                rows.append({"case": "ks divide study nx=2^%d" % e, "precision": prec,
                             "form": "divide" if flags else "multiply", "nx": nx, "steps": steps,
                             "us_per_step": us, "cell_updates_per_s": nx * steps / (res.kernel_ms * 1e-3)})
            rows[-2]["equal_to_multiply"] = bool(np.array_equal(outs[0], outs[1]))
            print("ks divide study nx=2^%-2d f%-2d divide %9.3f us/step  multiply %9.3f us/step  x%.2f  %s" % (
                e, prec * 8, line[-2], line[-1], line[-2] / line[-1],
                "bit-identical" if rows[-2]["equal_to_multiply"] else "DIFFERS"), flush=True)
        table.append(line)
    if path:
        Path(path).write_text("".join("%d\t%g\t%g\t%g\t%g\n" % tuple(t) for t in table))
    return rows


def main():
    import numpy as np
    import torch

    ap = argparse.ArgumentParser()
    ap.add_argument("--quick", action="store_true")
    ap.add_argument("--ensemble", action="store_true", help="also run the ensemble (config 4) rows")
    ap.add_argument("--json", default=None)
    ap.add_argument("--only", default=None, help="run only cases whose label contains one of these comma-separated texts")
    ap.add_argument("--precision", type=int, default=None, choices=[4, 8], help="run only this precision")
    ap.add_argument("--threads", default="0", help="comma-separated threads per swept block (0 = default)")
    ap.add_argument("--tpb", default=None, help="comma-separated tile widths (default: each case's own)")
    ap.add_argument("--algs", default="classic,swept,variant", help="comma-separated subset of classic,swept,variant")
    ap.add_argument("--divide", nargs="?", const="", default=None, metavar="TABLE",
                    help="run only the KS division study; write its table to TABLE if given")
    args = ap.parse_args()
    sw = importlib.import_module("1dsweptcuda_gb300")
    solver = sw.Solver(0)
    stream = torch.cuda.current_stream()
    thread_list = [int(t) for t in args.threads.split(",")]
    algs = {"classic": sw.ALG_CLASSIC, "swept": sw.ALG_SWEPT, "variant": sw.ALG_VARIANT}
    alg_list = [algs[a] for a in args.algs.split(",")]
    rows = []
    if args.divide is not None:
        rows = divide_rows(sw, solver, args.quick, args.divide or None)
        solver.close()
        if args.json:
            Path(args.json).write_text(json.dumps(rows, indent=1))
        return
    for label, prob, prec, bc, nx, tpbs, steps, dt in cases(args.quick):
        if (args.only and not any(o in label for o in args.only.split(","))) or \
                (args.precision and args.precision != prec):
            continue
        results = {}
        if args.tpb:
            tpbs = [int(t) for t in args.tpb.split(",")]
        runs = [(sw.ALG_CLASSIC, tpbs[0], 0)] if sw.ALG_CLASSIC in alg_list else []
        runs += [(alg, tpb, th) for tpb in tpbs for th in thread_list for alg in (sw.ALG_SWEPT, sw.ALG_VARIANT)
                 if alg in alg_list]
        for alg, tpb, th in runs:
            cfg = sw.make_config(prob, prec, alg=alg, nx=nx, tpb=tpb, dt=dt, bc=bc,
                                 time_mode=sw.TIME_STEPS, n_steps=steps)
            cfg.threads = th
            ic = sw.initial_condition(cfg)
            if prob == 2:
                dev = np.zeros((nx, 4), dtype=ic.dtype)
                dev[:, :3] = ic.reshape(-1, 3)
                ic = dev.ravel()
            elif prob == 0 and bc == 2:
                x = np.arange(nx)
                ic = (50 + 100 * np.sin(2 * np.pi * x / nx)).astype(ic.dtype)
            st = torch.from_numpy(ic).cuda()
            solver.run_device(cfg, st.data_ptr(), stream.cuda_stream)  # warm
            st = torch.from_numpy(ic).cuda()
            torch.cuda.synchronize()
            res = solver.run_device(cfg, st.data_ptr(), stream.cuda_stream)
            out = st.cpu().numpy()
            ups = nx * steps / (res.kernel_ms * 1e-3)
            key = ("classic" if alg == 0 else "swept" if alg == 1 else "variant", tpb, th)
            results[key] = (ups, out, res)
            row = {"case": label, "precision": prec, "alg": key[0], "tpb": tpb if alg else None,
                   "threads": th if alg else None,
                   "tile": res.tile, "nx": nx, "steps": steps, "ms": res.kernel_ms,
                   "cell_updates_per_s": ups, "launches": res.launches,
                   "finite": bool(np.isfinite(out).all())}
            rows.append(row)
        base = results.get(("classic", tpbs[0], 0)) or next(iter(results.values()))
        for (name, tpb, th), (ups, out, res) in results.items():
            same = np.array_equal(out, base[1])
            for r in rows:
                if r["case"] == label and r["precision"] == prec and r["alg"] == name and \
                        (name == "classic" or (r["tpb"] == tpb and r["threads"] == th)):
                    r["equal_to_classic"] = bool(same)
                    r["over_classic"] = ups / base[0]
        for r in rows:
            if r["case"] == label and r["precision"] == prec:
                print("%-34s f%-2d %-8s tpb=%-5s thr=%-4s %10.3e cell-updates/s  x%.2f vs classic  %s" % (
                    label, prec * 8, r["alg"], r["tpb"], r["threads"] or "-", r["cell_updates_per_s"],
                    r.get("over_classic", 1.0),
                    ("bit-identical" if r.get("equal_to_classic") else "DIFFERS") if sw.ALG_CLASSIC in alg_list
                    else ""), flush=True)
    if args.ensemble:
        rows += ensemble_rows(sw, solver, args.quick)
    solver.close()
    if args.json:
        Path(args.json).write_text(json.dumps(rows, indent=1))


if __name__ == "__main__":
    main()
