"""Accuracy of the benchmark configurations against their references, on the
GPU (run with -s for the tables):

* KS FP64, config 2 (periodic, dx = 0.5, dt = 0.005, the reference IC): the
  swept solution against a dt = 1e-5 FP64 run of the same scheme (the small
  time-step oracle), on the 2^14-cell window the IC repeats with -- from the
  tiled IC the 2^20 run is that window's run tiled, bit for bit, which the
  test also checks.  KS is chaotic, so the error is stated per time rather
  than bounded at tf = 200.
* Heat FP64, config 1 (periodic, Fo = 0.1, sine IC): against the exact
  discrete solution and the continuous one.
* Euler/Sod FP64: density L1 error against the exact Riemann solution at
  t = 0.2 for three resolutions.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KS, HEAT, EULER = 1, 0, 2
TIME_STEPS = 1


def _advance(sw, solver, problem, nx, tpb, dt, u, steps, **kw):
    cfg = sw.make_config(problem, 8, alg=sw.ALG_SWEPT, nx=nx, tpb=tpb, dt=dt, time_mode=TIME_STEPS, n_steps=steps,
                         **kw)
    fin, res, _ = solver.run(cfg, u)
    assert res.n_steps == steps
    return fin


def test_ks_against_small_time_step(sw, solver):
    window = 1 << 14
    times = [0.5, 1, 2, 5, 10, 20, 50, 100, 200]
    ic = sw.initial_condition(sw.make_config(KS, 8, nx=window))

    def trajectory(dt, tpb):
        u, done, out = ic.copy(), 0, []
        for t in times:
            n = int(round(t / dt)) - done
            u = _advance(sw, solver, KS, window, tpb, dt, u, n)
            done += n
            out.append(u.copy())
        return out

    run = trajectory(0.005, 256)
    ref = trajectory(1e-5, 1024)
    print("\nKS FP64, dx = 0.5, dt = 0.005 vs dt = 1e-5 (nx = 2^14 window of the 2^20 benchmark domain)")
    print("%8s %12s %12s %10s" % ("t", "rel-L2", "max |diff|", "max |u|"))
    rel = []
    for t, a, b in zip(times, run, ref):
        r = float(np.linalg.norm(a - b) / np.linalg.norm(b))
        rel.append(r)
        print("%8g %12.3e %12.3e %10.4f" % (t, r, float(np.abs(a - b).max()), float(np.abs(b).max())))
    assert all(np.isfinite(x) for x in rel)
    # second order in time before chaos amplifies the error: halving dt quarters it at t = 0.5
    half = _advance(sw, solver, KS, window, 256, 0.0025, ic.copy(), int(round(times[0] / 0.0025)))
    r_half = float(np.linalg.norm(half - ref[0]) / np.linalg.norm(ref[0]))
    print("t = 0.5: rel-L2 %.3e at dt = 0.005, %.3e at dt = 0.0025 (ratio %.2f)" % (rel[0], r_half, rel[0] / r_half))
    assert 3.0 < rel[0] / r_half < 5.0, (rel[0], r_half)

    # The benchmark's 2^20-cell IC is the window tiled 64 times up to the rounding
    # of the cosine's argument at large x (<= 1e-10), and from the tiled IC the
    # 2^20 run is the window's run tiled, bit for bit.
    big_ic = sw.initial_condition(sw.make_config(KS, 8, nx=1 << 20))
    assert float(np.abs(big_ic - np.tile(ic, 64)).max()) < 1e-10
    big = _advance(sw, solver, KS, 1 << 20, 256, 0.005, np.tile(ic, 64), int(round(times[0] / 0.005)))
    np.testing.assert_array_equal(big, np.tile(run[0], 64))


def test_heat_config1_against_exact(sw, solver):
    from oracle import exact
    nx, tpb, steps = 4096, 128, 20000
    dt = 0.1 * 0.001 ** 2 / 8.418e-5
    x = np.arange(nx)
    ic = 50 + 100 * np.sin(2 * np.pi * x / nx)
    cfg = sw.make_config(HEAT, 8, alg=sw.ALG_SWEPT, nx=nx, tpb=tpb, dt=dt, bc=sw.BC_PERIODIC, time_mode=TIME_STEPS,
                         n_steps=steps)
    k = sw.constants(cfg)
    fin, _, _ = solver.run(cfg, ic)
    disc = exact.heat_periodic_mode(steps, nx, k.fourier, fourier_two=k.fourier_two)
    cont = exact.heat_periodic_mode(steps, nx, k.fourier, discrete=False)
    e_disc, e_cont = float(np.abs(fin - disc).max()), float(np.abs(fin - cont).max())
    print("\nHeat FP64 periodic, nx = 4096, Fo = %.6g, %d steps: max |err| vs exact discrete %.3e, "
          "vs continuous %.3e (amplitude %.3f)" % (k.fourier, steps, e_disc, e_cont, float(np.abs(fin - 50).max())))
    assert e_disc < 1e-9 and e_cont < 1e-3


def test_sod_convergence(sw, solver):
    from oracle import exact
    print("\nEuler/Sod FP64 swept, t = 0.2, dt = 0.1 dx: density L1 error vs the exact Riemann solution")
    errs = []
    for nx, tpb in ((1024, 32), (4096, 64), (16384, 64)):  # nx points including the two Dirichlet cells
        dt = 0.1 / (nx - 2)
        steps = int(round(0.2 / dt))
        cfg = sw.make_config(EULER, 8, alg=sw.ALG_SWEPT, nx=nx, tpb=tpb, dt=dt, time_mode=TIME_STEPS, n_steps=steps)
        fin, _, _ = solver.run(cfg)
        q = fin.reshape(-1, 3)
        ex = exact.sod(exact.sod_cell_centres(nx), steps * dt)
        e = float(np.mean(np.abs(q[1:-1, 0] - ex["density"])))
        errs.append(e)
        print("  nx = %6d: L1 %.3e" % (nx, e))
    assert errs[0] > errs[1] > errs[2] and errs[1] < 1e-3


def test_ks_dt_sweep_against_reference_golden(sw, solver, golden):
    """The reference's own accuracy procedure for KS (testProcedure.py:242-253:
    nx = 1024, tpb = 64, dt from 1e-4 down) against its golden run
    (Testing/KSDouble_Official.txt: FP64 swept, dt = 1e-7) at t = 6, with three
    larger steps added where the scheme's O(dt^2) error is above the file's
    10-digit resolution (~5e-10 at |u| < 10)."""
    g = golden["ks"]
    want = g["velocity"][1]
    assert float(g["times"][1]) == 6.0
    dts = (2e-3, 1e-3, 5e-4, 1e-4, 5e-5, 1e-5)
    errs = []
    print("\nKS FP64 swept, nx = 1024, tpb = 64, t = 6, against the reference's golden run (dt = 1e-7)")
    for dt in dts:
        cfg = sw.make_config(KS, 8, nx=1024)
        ic = sw.initial_condition(cfg)
        u = _advance(sw, solver, KS, 1024, 64, dt, ic, int(round(6.0 / dt)))
        e = float(np.abs(u - want).max())
        errs.append(e)
        print("  dt = %-6g max |err| %.3e" % (dt, e))
    for a, b in zip(errs[:2], errs[1:3]):
        assert 3.0 < a / b < 5.0, errs  # second order in dt
    assert max(errs[3:]) < 1.5e-9, errs  # at the golden file's resolution
