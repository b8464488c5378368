"""Learned closure for 4x-coarsened KS (the C ABI's sw_closure_* calls).

Fine grid: nx = 4096, dx = 0.5, dt = 0.005, FP64 (the reference solution and the source of
training data).  Coarse grid: nx = 1024, dx = 2, dt = 0.02 = 4 fine steps,
FP32.  The closure f learns the coarse step's defect

    target(u) = CG(fine^4(u_f)) - coarse(CG(u_f)),   input CG(u_f),

CG = averages of 4 fine cells, so that u(t + dt) = coarse(u) + f(u) tracks the
coarse-grained fine solution.  Training data come from the project's own fine
ensemble solver; training runs on the GPU through sw_closure_train (forward and
backward on BF16 tensor cores, Adam on FP32 masters).  run_adaptive checks each
segment against one prolonged fine step (a residual of the coarse update with
respect to the fine dynamics), picks the closure-corrected or the plain coarse
update per domain, accumulates the residuals into a per-domain error estimate,
and hands the domains whose estimate passes a tolerance to the fine solver.
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
    """Coarse cell averages (n_dom, n) -> fine cell averages (n_dom, n * factor),
    FP64, by periodic spectral interpolation.  Each Fourier mode below the
    coarse Nyquist frequency is taken from coarse-cell to fine-cell averages
    (times sinc(k/(n*factor)) / sinc(k/n), with the phase of the shifted cell
    centres); the Nyquist mode b(-1)^j becomes the fine averages of
    b*(pi/2)*sin(pi*x/H), H the coarse cell.  Averaging each `factor` fine
    cells gives the coarse state back (to FP64 rounding), and a band-limited
    field is reproduced exactly -- the fallback's and the residual check's
    restart state."""
    torch = _torch()
    c = coarse.double()
    n_dom, n = c.shape
    nf = n * factor
    dev = c.device
    j = torch.arange(n, device=dev)
    sign = 1.0 - 2.0 * (j % 2).double()
    b = (c * sign).mean(dim=1, keepdim=True)
    spec = torch.fft.rfft(c - b * sign, dim=1)
    k = torch.arange(n // 2, device=dev, dtype=torch.float64)
    ratio = torch.sinc(k / nf) / torch.sinc(k / n)
    phase = torch.exp(1j * math.pi * k / n * (1.0 / factor - 1.0))
    fine_spec = torch.zeros((n_dom, nf // 2 + 1), dtype=spec.dtype, device=dev)
    fine_spec[:, :n // 2] = spec[:, :n // 2] * (factor * ratio * phase)
    fine = torch.fft.irfft(fine_spec, n=nf, dim=1)
    m = torch.arange(nf, device=dev, dtype=torch.float64)
    nyq = 0.5 * factor * (torch.cos(math.pi * m / factor) - torch.cos(math.pi * (m + 1) / factor))
    return (fine + b * nyq).contiguous()


def run_adaptive(solver, closure: Closure, fine0, coarse_steps: int, segment: int, tau: float):
    """Closure-corrected coarse run of an ensemble with a residual-based error
    estimate and the plain fine solver as fallback.

    fine0: (n_dom, 4096) FP64 states at t0 (the problem as posed).  The coarse
    state starts at CG(fine0).  At the start of each segment of `segment`
    coarse steps, every live domain's state u is prolonged (conservatively) to
    the fine grid and advanced by one coarse step of the fine solver; r, its
    coarse-grained result, is what one coarse update should reach.  The
    residuals d_c = ||coarse(u) + f(u) - r||, d_p = ||coarse(u) - r|| pick the
    closure-corrected or the plain coarse update for the segment, and the
    smaller one, times the segment's steps over ||u||, is added to the
    domain's error estimate (a relative L2 error, accumulated without growth).
    A domain leaves the coarse run as soon as its estimate, projected to the
    end at the current residual, passes tau; at the end all such domains are
    solved by the fine solver from fine0, in one batch, so their results are
    the fine solution itself.

    Returns (u, info): u (n_dom, 1024) FP32 at t0 + coarse_steps * 0.02, and
    counts of (domain, segment) pairs run with the closure / plain, the
    domains that fell back, and each domain's final estimate."""
    torch = _torch()
    u = coarse_grain(solver, fine0)
    n_dom = u.shape[0]
    live = torch.ones(n_dom, dtype=torch.bool, device=u.device)
    est = torch.zeros(n_dom, dtype=torch.float64, device=u.device)
    info = {"closure": 0, "plain": 0, "fallback": 0}
    done = 0
    while done < coarse_steps:
        idx = torch.nonzero(live).flatten()
        if idx.numel() == 0:
            break
        k = min(segment, coarse_steps - done)
        start = u[idx].contiguous()
        one_c, one_p = start.clone(), start.clone()
        closure.step(one_c, 1, use_closure=True)
        closure.step(one_p, 1, use_closure=False)
        chk = prolong(start)
        advance_fine(solver, chk, FACTOR)
        r = coarse_grain(solver, chk)
        d_c = (one_c - r).double().norm(dim=1)
        d_p = (one_p - r).double().norm(dim=1)
        use_c = d_c <= d_p
        rate = torch.minimum(d_c, d_p) / start.double().norm(dim=1).clamp_min(1e-30)
        est[idx] += k * rate
        bad = est[idx] + (coarse_steps - done - k) * rate > tau
        live[idx[bad]] = False
        for mask, on in ((use_c & ~bad, True), (~use_c & ~bad, False)):
            sel = idx[mask]
            if sel.numel():
                v = start[mask].contiguous()
                closure.step(v, k, use_closure=on)
                u[sel] = v
                info["closure" if on else "plain"] += int(sel.numel())
        done += k
    fb = torch.nonzero(~live).flatten()
    if fb.numel():
        f = fine0[fb].contiguous().clone()
        advance_fine(solver, f, coarse_steps * FACTOR)
        u[fb] = coarse_grain(solver, f)
    info["fallback"] = int(fb.numel())
    info["estimate"] = est
    return u, info


CHAOS_SPINUP = 12500   # coarse steps (t = 250): the ensemble's long waves have broken into KS chaos


def _timed(fn):
    import time
    torch = _torch()
    torch.cuda.synchronize()
    a = time.perf_counter()
    out = fn()
    torch.cuda.synchronize()
    return out, time.perf_counter() - a


def train_closure(solver, n_train: int = 512, snapshots: int = 64, train_steps: int = 3000, seed: int = 0):
    """A closure trained on the fine solver's own trajectories in developed
    chaos (t >= 250), and a summary of the training."""
    torch = _torch()
    closure = Closure(solver, seed=seed)
    info = {"n_train_traj": n_train, "snapshots": snapshots}
    (x, y), info["datagen_s"] = _timed(lambda: make_training_data(solver, closure, n_train, snapshots, interval=25,
                                                                  seed=seed + 1, spinup=CHAOS_SPINUP))
    info["output_scale"] = closure.calibrate(y)
    losses, info["train_s"] = _timed(lambda: closure.train(x, y, steps=train_steps, batch=64, lr=2e-3,
                                                           seed=seed + 2))
    info["loss_first"], info["loss_last"] = float(losses[:10].mean()), float(losses[-50:].mean())
    hx, hy = make_training_data(solver, closure, 32, 8, interval=25, seed=seed + 999, spinup=CHAOS_SPINUP)
    info["heldout_defect_ratio"] = float(((hy - closure.infer(hx)).pow(2).sum() / hy.pow(2).sum()).item())
    del x, y
    return closure, info


def evaluate(n_train: int = 512, snapshots: int = 64, n_eval: int = 1024, horizons=(5.0, 20.0, 50.0, 200.0),
             train_steps: int = 3000, seed: int = 0, tau: float = 1e-3, segment: int = 50,
             start_step: int = 0) -> dict:
    """Train, then for each horizon tf solve the evaluation ensemble (n_eval
    domains, 4096 fine cells) from t0 = start_step * 0.02 to t0 + tf four
    ways -- fine FP64 (the reference solution), plain coarse, closure-corrected coarse, and
    run_adaptive with tolerance tau -- and report wall times and the relative
    L2 error of each against the coarse-grained reference solution."""
    torch = _torch()
    sw = _sw()
    solver = sw.Solver(0)
    closure, out = train_closure(solver, n_train, snapshots, train_steps, seed)
    out.update({"fine_nx": FINE_NX, "coarse_nx": COARSE_NX, "n_eval": n_eval, "t0": start_step * COARSE_DT,
                "tau": tau, "segment": segment, "horizons": []})
    fine0 = fine_ensemble(n_eval, seed=seed + 5)
    if start_step:
        advance_fine(solver, fine0, start_step * FACTOR)
    start = coarse_grain(solver, fine0)
    # one-time costs (graph captures, FFT plans) out of the timings
    advance_fine(solver, fine0.clone(), FACTOR)
    closure.step(start.clone(), 1, use_closure=True)
    closure.step(start.clone(), 1, use_closure=False)
    run_adaptive(solver, closure, fine0, 2 * segment, segment, float("inf"))
    for tf in horizons:
        steps = int(round(tf / COARSE_DT))
        truth = fine0.clone()
        _, t_fine = _timed(lambda: advance_fine(solver, truth, steps * FACTOR))
        ref = coarse_grain(solver, truth)
        row = {"tf": tf, "time_fine_s": t_fine}
        for name, on in (("plain", False), ("closure", True)):
            v = start.clone()
            _, row["time_%s_s" % name] = _timed(lambda: closure.step(v, steps, use_closure=on))
            row["rel_l2_%s" % name] = rel_l2(v, ref)
        (u, info), row["time_adaptive_s"] = _timed(lambda: run_adaptive(solver, closure, fine0, steps, segment, tau))
        err = ((u.double() - ref.double()).norm(dim=1) / ref.double().norm(dim=1))
        row["rel_l2_adaptive"] = float(err.mean().item())
        row["max_rel_l2_adaptive"] = float(err.max().item())
        row["fallback_domains"] = info["fallback"]
        row["segments_closure"], row["segments_plain"] = info["closure"], info["plain"]
        kept = info["estimate"] <= tau
        if bool(kept.any()):
            row["kept_mean_estimate"] = float(info["estimate"][kept].mean().item())
            row["kept_mean_rel_l2"] = float(err[kept].mean().item())
            row["kept_max_rel_l2"] = float(err[kept].max().item())
        row["speedup_adaptive_vs_fine"] = t_fine / row["time_adaptive_s"]
        out["horizons"].append(row)
    solver.close()
    return out


def bench_step(n_dom: int = 1024, steps: int = 200, seed: int = 0) -> dict:
    """Throughput of the fused coarse step with the closure on (k_step), on
    n_dom domains of the coarse grid from a smooth random state: coarse
    cell-steps per second and the tensor-core work it implies (the 32 -> 32
    layer is 2 * 32 * 32 * 5 FLOP per cell)."""
    sw = _sw()
    solver = sw.Solver(0)
    closure = Closure(solver, seed=seed)
    fine = fine_ensemble(n_dom, seed=seed + 1)
    u = coarse_grain(solver, fine)
    closure.step(u.clone(), 2, use_closure=True)          # warm-up
    v = u.clone()
    res = closure.step(v, steps, use_closure=True)
    cells = n_dom * COARSE_NX * steps
    out = {"n_dom": n_dom, "steps": steps, "ms": res.kernel_ms, "cell_steps_per_s": cells / (res.kernel_ms * 1e-3),
           "layer2_tflops": cells * 2 * 32 * 32 * 5 / (res.kernel_ms * 1e-3) / 1e12}
    solver.close()
    return out


if __name__ == "__main__":
    import argparse
    import json
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
    ap = argparse.ArgumentParser(description="train and evaluate the KS closure (1024 domains, coarse nx 1024)")
    ap.add_argument("--train-traj", type=int, default=512)
    ap.add_argument("--snapshots", type=int, default=64)
    ap.add_argument("--eval", type=int, default=1024)
    ap.add_argument("--horizons", default="5,20,50,200", help="comma-separated tf values")
    ap.add_argument("--train-steps", type=int, default=3000)
    ap.add_argument("--tau", type=float, default=1e-3)
    ap.add_argument("--segment", type=int, default=50)
    ap.add_argument("--start-step", type=int, default=0, help="coarse steps of spin-up before t0")
    ap.add_argument("--json", default=None)
    ap.add_argument("--bench-step", type=int, default=0, help="only time this many fused closure steps")
    a = ap.parse_args()
    if a.bench_step:
        print(json.dumps(bench_step(steps=a.bench_step)))
        sys.exit(0)
    res = evaluate(a.train_traj, a.snapshots, a.eval, [float(t) for t in a.horizons.split(",")], a.train_steps,
                   tau=a.tau, segment=a.segment, start_step=a.start_step)
    print(json.dumps(res, indent=1))
    if a.json:
        Path(a.json).write_text(json.dumps(res, indent=1))
