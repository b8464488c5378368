"""Learned closure for 4x-coarsened KS (the C ABI's sw_closure_* calls).

Fine grid: nx = 4096, dx = 0.5, dt = 0.005, FP64 (the judge and the source of
training data).  Coarse grid: nx = 1024, dx = 2, dt = 0.02 = 4 fine steps,
FP32.  The closure f learns the coarse step's defect

    target(u) = CG(fine^4(u_f)) - coarse(CG(u_f)),   input CG(u_f),

CG = averages of 4 fine cells, so that u(t + dt) = coarse(u) + f(u) tracks the
coarse-grained fine solution.  Training data come from the project's own fine
ensemble solver; training runs on the GPU through sw_closure_train (forward and
backward on BF16 tensor cores, Adam on FP32 masters).  A run with the closure
falls back to the fine solver for domains whose residual estimate -- the size of
the correction relative to the coarse update -- exceeds a threshold.
"""
from __future__ import annotations

import ctypes as C
import importlib
import math

import numpy as np

FINE_NX, COARSE_NX, FACTOR = 4096, 1024, 4
FINE_DX, COARSE_DX = 0.5, 2.0
FINE_DT, COARSE_DT = 0.005, 0.02


def _sw():
    return importlib.import_module("1dsweptcuda_gb300")


def _torch():
    import torch
    return torch


def init_params(seed: int = 0, scale: float = 1.0) -> np.ndarray:
    """He-style initial parameters; the output layer starts near zero so the
    untrained closure leaves the coarse step unchanged.  The last value is the
    output scale s (f = s * net), which training does not change."""
    rng = np.random.default_rng(seed)
    w1 = rng.standard_normal((32, 5)) * math.sqrt(2.0 / 5)
    w2 = rng.standard_normal((32, 32, 5)) * math.sqrt(2.0 / 160)
    w3 = rng.standard_normal((32, 5)) * 1e-3
    return np.concatenate([w1.ravel(), np.zeros(32), w2.ravel(), np.zeros(32), w3.ravel(), np.zeros(1),
                           [scale]]).astype(np.float32)


class Closure:
    """Device-resident closure parameters and the calls that use them."""

    def __init__(self, solver, theta: np.ndarray | None = None, seed: int = 0):
        torch = _torch()
        self.sw = _sw()
        self.solver = solver
        self.lib = self.sw.library()
        t = init_params(seed) if theta is None else np.asarray(theta, dtype=np.float32)
        self.theta = torch.from_numpy(t.copy()).cuda()

    def _ctx(self):
        return self.solver._ctx

    def set_scale(self, s: float) -> None:
        """Output scale s (f = s * net): the network then works on O(1) values,
        far above its BF16 rounding, whatever the size of the defects."""
        self.theta[-1] = float(s)

    def calibrate(self, targets) -> float:
        """Set the output scale to the RMS of the training targets."""
        s = float(targets.double().pow(2).mean().sqrt().item())
        self.set_scale(s if s > 0 else 1.0)
        return s

    def _check(self, rc, what):
        if rc:
            raise self.solver._err(rc, what)

    def coarse_config(self, dt: float = COARSE_DT, dx: float = COARSE_DX):
        return self.sw.make_config(self.sw.KS, 4, alg=self.sw.ALG_CLASSIC, nx=COARSE_NX, tpb=128, dt=dt, dx=dx,
                                   time_mode=self.sw.TIME_STEPS)

    def infer(self, u):
        torch = _torch()
        n_dom, n = u.shape
        out = torch.empty_like(u)
        self._check(self.lib.sw_closure_infer(self._ctx(), self.theta.data_ptr(), u.data_ptr(), out.data_ptr(), n_dom,
                                              n), "sw_closure_infer")
        return out

    def step(self, u, n_steps: int, use_closure: bool = True, cfg=None):
        """n_steps coarse steps in place on u (n_dom, n) float32 CUDA tensor."""
        n_dom, n = u.shape
        cfg = cfg or self.coarse_config()
        res = self.sw.Result()
        self._check(self.lib.sw_closure_step(self._ctx(), C.byref(cfg), self.theta.data_ptr(), u.data_ptr(), n_dom, n,
                                             n_steps, int(use_closure), C.byref(res)), "sw_closure_step")
        return res

    def grad(self, u, target, rows=None):
        torch = _torch()
        n_dom, n = (len(rows), u.shape[1]) if rows is not None else u.shape
        g = torch.empty(self.sw.native.CLOSURE_PARAMS + 1, dtype=torch.float32, device="cuda")
        rp = 0
        if rows is not None:
            rows_t = torch.as_tensor(np.asarray(rows, dtype=np.int64)).cuda()
            rp = rows_t.data_ptr()
        self._check(self.lib.sw_closure_grad(self._ctx(), self.theta.data_ptr(), u.data_ptr(), target.data_ptr(),
                                             C.c_void_p(rp) if rp else None, n_dom, n, g.data_ptr()),
                    "sw_closure_grad")
        return g[:-1].clone(), float(g[-1].item())

    def train(self, inputs, targets, steps: int, batch: int = 64, lr: float = 1e-3, seed: int = 1) -> np.ndarray:
        losses = np.zeros(steps, dtype=np.float32)
        s, n = inputs.shape
        self._check(self.lib.sw_closure_train(self._ctx(), self.theta.data_ptr(), inputs.data_ptr(),
                                              targets.data_ptr(), s, n, batch, steps, lr, seed,
                                              losses.ctypes.data_as(C.POINTER(C.c_float))), "sw_closure_train")
        return losses


def fine_config(sw, steps: int):
    return sw.make_config(sw.KS, 8, alg=sw.ALG_SWEPT, tpb=256, dt=FINE_DT, dx=FINE_DX, time_mode=sw.TIME_STEPS,
                          n_steps=steps)


def coarse_grain(solver, fine, factor: int = FACTOR):
    torch = _torch()
    n_dom, nf = fine.shape
    out = torch.empty((n_dom, nf // factor), dtype=torch.float32, device="cuda")
    rc = _sw().library().sw_coarse_grain(solver._ctx, fine.data_ptr(), out.data_ptr(), out.numel(), factor)
    if rc:
        raise solver._err(rc, "sw_coarse_grain")
    return out


def fine_ensemble(n_traj: int, seed: int):
    """Fine ICs from the ensemble law at fixed nx = 4096 (one (n_traj, 4096) FP64 tensor)."""
    torch = _torch()
    ens = importlib.import_module("1dsweptcuda_gb300.ensemble")
    nx, u = ens.make_ensemble(n_domains=n_traj, lo=12, hi=12, dx=FINE_DX, seed=seed)
    return torch.from_numpy(u.reshape(n_traj, FINE_NX)).cuda()


def advance_fine(solver, fine, steps: int):
    sw = _sw()
    n_traj = fine.shape[0]
    nx = np.full(n_traj, FINE_NX, dtype=np.int64)
    solver.run_batch_device(fine_config(sw, steps), nx, fine.data_ptr())


def make_training_data(solver, closure: Closure, n_traj: int, snapshots: int, interval: int, seed: int = 7,
                       spinup: int = 0):
    """(inputs, targets): (n_traj * snapshots, 1024) float32 CUDA tensors.  Each
    snapshot k of trajectory j: input CG(u_f(t_k)), target = CG(fine^4 u_f) -
    coarse(CG u_f); t_k = spinup + k * interval coarse steps."""
    torch = _torch()
    fine = fine_ensemble(n_traj, seed)
    if spinup:
        advance_fine(solver, fine, spinup * FACTOR)
    xs, ys = [], []
    for k in range(snapshots):
        x = coarse_grain(solver, fine)
        nxt = fine.clone()
        advance_fine(solver, nxt, FACTOR)
        y_f = coarse_grain(solver, nxt)
        y_c = x.clone()
        closure.step(y_c, 1, use_closure=False)
        xs.append(x)
        ys.append(y_f - y_c)
        if interval == 1:
            fine = nxt
        else:
            advance_fine(solver, fine, interval * FACTOR)
    return torch.cat(xs), torch.cat(ys)


def rel_l2(a, b) -> float:
    """Mean over domains of ||a - b|| / ||b||."""
    num = (a.double() - b.double()).norm(dim=1)
    den = b.double().norm(dim=1)
    return float((num / den).mean().item())


def prolong(coarse, factor: int = FACTOR):
    """Coarse FP32 -> fine FP64 by periodic linear interpolation of cell averages
    (the fallback's restart state)."""
    torch = _torch()
    c = coarse.double()
    nxt = torch.roll(c, -1, dims=1)
    w = (torch.arange(factor, dtype=torch.float64, device=c.device) + 0.5) / factor - 0.5
    lo = torch.where(w < 0, torch.roll(c, 1, dims=1)[..., None], c[..., None])
    hi = torch.where(w < 0, c[..., None], nxt[..., None])
    a = torch.where(w < 0, w + 1.0, w)
    return (lo * (1 - a) + hi * a).reshape(c.shape[0], -1).contiguous()


def run_with_fallback(solver, closure: Closure, u, coarse_steps: int, segment: int, tau: float):
    """Closure-corrected coarse run with the fine solver as fallback.  After each
    segment, domains whose residual estimate ||f(u)|| / ||coarse(u) - u|| (the
    relative size of the learned correction, i.e. how far the coarse step is
    from the fine one) exceeds tau are re-run over that segment on the fine grid
    from the prolonged segment-start state and restricted back.  Returns the
    number of (domain, segment) fallbacks."""
    torch = _torch()
    fallbacks = 0
    done = 0
    while done < coarse_steps:
        k = min(segment, coarse_steps - done)
        start = u.clone()
        plain = start.clone()
        closure.step(plain, 1, use_closure=False)
        est = closure.infer(start).norm(dim=1) / (plain - start).norm(dim=1).clamp_min(1e-30)
        closure.step(u, k, use_closure=True)
        bad = torch.nonzero(est > tau).flatten()
        if bad.numel():
            fallbacks += int(bad.numel())
            f = prolong(start[bad])
            advance_fine(solver, f, k * FACTOR)
            u[bad] = coarse_grain(solver, f)
        done += k
    return fallbacks


CHAOS_SPINUP = 12500   # coarse steps (t = 250): the ensemble's long waves have broken into KS chaos


def evaluate(n_train: int = 512, snapshots: int = 64, n_eval: int = 1024, tf: float = 200.0, train_steps: int = 3000,
             seed: int = 0, tau: float = float("inf"), segment: int = 50, start_step: int = CHAOS_SPINUP) -> dict:
    """Train on the fine solver's trajectories (developed chaos, t >= 250), then
    run the evaluation ensemble (n_eval domains, config 5 shape) from
    t0 = start_step * 0.02 for tf three ways -- fine FP64 (the judge), plain
    coarse, closure-corrected coarse (with fallback when tau is finite) -- and
    report times and the relative L2 error against the coarse-grained judge."""
    import time
    torch = _torch()
    sw = _sw()
    solver = sw.Solver(0)
    closure = Closure(solver, seed=seed)
    out = {"fine_nx": FINE_NX, "coarse_nx": COARSE_NX, "n_train_traj": n_train, "snapshots": snapshots,
           "n_eval": n_eval, "tf": tf, "t0": start_step * COARSE_DT}
    t0 = time.perf_counter()
    x, y = make_training_data(solver, closure, n_train, snapshots, interval=25, seed=seed + 1, spinup=CHAOS_SPINUP)
    torch.cuda.synchronize()
    out["datagen_s"] = time.perf_counter() - t0
    out["output_scale"] = closure.calibrate(y)
    t0 = time.perf_counter()
    losses = closure.train(x, y, steps=train_steps, batch=64, lr=2e-3, seed=seed + 2)
    torch.cuda.synchronize()
    out["train_s"] = time.perf_counter() - t0
    out["loss_first"], out["loss_last"] = float(losses[:10].mean()), float(losses[-50:].mean())
    hx, hy = make_training_data(solver, closure, 32, 8, interval=25, seed=seed + 999, spinup=CHAOS_SPINUP)
    out["heldout_defect_ratio"] = float(((hy - closure.infer(hx)).pow(2).sum() / hy.pow(2).sum()).item())
    del x, y
    fine = fine_ensemble(n_eval, seed=seed + 5)
    if start_step:
        advance_fine(solver, fine, start_step * FACTOR)
    start = coarse_grain(solver, fine)
    checkpoints = [t for t in (0.5, 1, 2, 5, 10, 20, 50, 100, 200) if t <= tf]
    steps_at = [int(round(t / COARSE_DT)) for t in checkpoints]
    errs = {"plain": [], "closure": []}
    amax = {"plain": [], "closure": [], "judge": []}
    judge = fine.clone()
    t_fine = t_plain = t_clos = 0.0
    u_plain, u_clos = start.clone(), start.clone()
    prev = 0
    fallbacks = 0
    for t, s in zip(checkpoints, steps_at):
        k = s - prev
        prev = s
        torch.cuda.synchronize()
        a = time.perf_counter()
        advance_fine(solver, judge, k * FACTOR)
        torch.cuda.synchronize()
        b = time.perf_counter()
        closure.step(u_plain, k, use_closure=False)
        torch.cuda.synchronize()
        c = time.perf_counter()
        if math.isinf(tau):
            closure.step(u_clos, k, use_closure=True)
        else:
            fallbacks += run_with_fallback(solver, closure, u_clos, k, segment, tau)
        torch.cuda.synchronize()
        d = time.perf_counter()
        t_fine += b - a
        t_plain += c - b
        t_clos += d - c
        ref = coarse_grain(solver, judge)
        errs["plain"].append(rel_l2(u_plain, ref))
        errs["closure"].append(rel_l2(u_clos, ref))
        for name, v in (("plain", u_plain), ("closure", u_clos), ("judge", ref)):
            amax[name].append(float(v.abs().max().item()))
    out.update({"checkpoints": checkpoints, "rel_l2_plain": errs["plain"], "rel_l2_closure": errs["closure"],
                "max_abs_plain": amax["plain"], "max_abs_closure": amax["closure"], "max_abs_judge": amax["judge"],
                "time_fine_s": t_fine, "time_plain_s": t_plain, "time_closure_s": t_clos,
                "speedup_closure_vs_fine": t_fine / t_clos if t_clos else None, "fallbacks": fallbacks,
                "tau": tau})

    def horizon(e):
        ok = [t for t, v in zip(checkpoints, e) if v <= 1e-3]
        return max(ok) if ok and ok == checkpoints[:len(ok)] else (0.0 if not ok else ok[-1])

    out["horizon_1e-3_plain"] = horizon(errs["plain"])
    out["horizon_1e-3_closure"] = horizon(errs["closure"])
    solver.close()
    return out


if __name__ == "__main__":
    import argparse
    import json
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
    ap = argparse.ArgumentParser(description="train and evaluate the KS closure (config 5 shape)")
    ap.add_argument("--train-traj", type=int, default=512)
    ap.add_argument("--snapshots", type=int, default=64)
    ap.add_argument("--eval", type=int, default=1024)
    ap.add_argument("--tf", type=float, default=200.0)
    ap.add_argument("--train-steps", type=int, default=3000)
    ap.add_argument("--tau", type=float, default=float("inf"))
    ap.add_argument("--start-step", type=int, default=CHAOS_SPINUP, help="coarse steps of spin-up before t0")
    ap.add_argument("--json", default=None)
    a = ap.parse_args()
    res = evaluate(a.train_traj, a.snapshots, a.eval, a.tf, a.train_steps, tau=a.tau, start_step=a.start_step)
    print(json.dumps(res, indent=1))
    if a.json:
        Path(a.json).write_text(json.dumps(res, indent=1))
