"""Full-size GPU checks through size-independent properties: at the benchmark
sizes the oracle would take minutes, so swept / variant are compared with the
classic kernel bit for bit (each is independently bit-identical to the oracle
at small sizes), and the periodic heat run is compared with the scheme's exact
discrete solution."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(sw, solver, torch, problem, prec, alg, nx, tpb, dt, steps, ic, bc=0):
    cfg = sw.make_config(problem, prec, alg=alg, nx=nx, tpb=tpb, dt=dt, bc=bc, time_mode=sw.TIME_STEPS,
                         n_steps=steps)
    st = torch.from_numpy(ic.copy()).cuda()
    res = solver.run_device(cfg, st.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert res.n_steps == steps
    return st.cpu().numpy()


def test_ks_benchmark_config_swept_equals_classic(sw, solver):
    """KS FP64, nx=2^20, tpb=256, dt=0.005, tf=200 (40000 steps): swept == classic."""
    torch = pytest.importorskip("torch")
    nx, tpb, dt, steps = 1 << 20, 256, 0.005, 40000
    ic = sw.initial_condition(sw.make_config(1, 8, nx=nx, tpb=tpb, dt=dt))
    a = _run(sw, solver, torch, 1, 8, sw.ALG_SWEPT, nx, tpb, dt, steps, ic)
    b = _run(sw, solver, torch, 1, 8, sw.ALG_CLASSIC, nx, tpb, dt, steps, ic)
    assert np.isfinite(a).all()
    np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("prec", [8, 4])
def test_heat_periodic_mode_exact_discrete(sw, solver, prec):
    """Heat periodic, nx=4096, tpb=128, Fo=0.1, IC 100 sin(2 pi x/L)+50, 20000
    steps: every path equals the scheme's exact discrete solution (computed with
    the run's rounded Fo and 1-2Fo) within 1e-12 relative in FP64 and 1e-3 in
    FP32 (20000 steps of float rounding drift by 3.8e-4 on GB300), and in FP64
    the continuous decay within 1e-3."""
    torch = pytest.importorskip("torch")
    from oracle import exact
    nx, tpb = 4096, 128
    dt = 0.1 * 0.001 ** 2 / 8.418e-5
    cfg = sw.make_config(0, prec, alg=sw.ALG_SWEPT, nx=nx, tpb=tpb, dt=dt, bc=sw.BC_PERIODIC)
    fo = sw.constants(cfg).fourier
    x = np.arange(nx)
    ic = (50 + 100 * np.sin(2 * np.pi * x / nx)).astype(np.float64 if prec == 8 else np.float32)
    steps = 20000
    for alg in (sw.ALG_SWEPT, sw.ALG_VARIANT, sw.ALG_CLASSIC):
        u = _run(sw, solver, torch, 0, prec, alg, nx, tpb, dt, steps, ic, bc=2).astype(np.float64)
        want = exact.heat_periodic_mode(steps, nx, fo, fourier_two=sw.constants(cfg).fourier_two)
        rel = np.abs(u - want).max() / np.abs(want).max()
        assert rel < (1e-12 if prec == 8 else 1e-3), (alg, rel)
        if prec == 8:
            cont = exact.heat_periodic_mode(steps, nx, fo, discrete=False)
            assert np.abs(u - cont).max() < 1e-3


@pytest.mark.parametrize("prec", [8, 4])
def test_euler_2_22_swept_equals_classic(sw, solver, prec):
    """Euler Sod, nx=2^22, tpb=512, dt/dx=0.1: swept and variant == classic over 256 steps."""
    torch = pytest.importorskip("torch")
    nx, tpb = 1 << 22, 512
    dt = 0.1 / (nx - 2)
    cfg = sw.make_config(2, prec, nx=nx, tpb=tpb, dt=dt)
    ic3 = sw.initial_condition(cfg).reshape(-1, 3)
    ic = np.zeros((nx, 4), dtype=ic3.dtype)
    ic[:, :3] = ic3
    ic = ic.ravel()
    b = _run(sw, solver, torch, 2, prec, sw.ALG_CLASSIC, nx, tpb, dt, 256, ic)
    for alg in (sw.ALG_SWEPT, sw.ALG_VARIANT):
        a = _run(sw, solver, torch, 2, prec, alg, nx, tpb, dt, 256, ic)
        np.testing.assert_array_equal(a, b)
    assert np.isfinite(b).all()


def test_sod_accuracy_gpu(sw, solver):
    """Swept Euler FP64 on the GPU reaches t = 0.2 with density L1 error < 0.001
    against the exact Riemann solution at 4094 interior cells (the oracle's
    classic run gives 7.9e-4 there and 2.1e-3 at 1024 cells)."""
    from oracle import exact
    nx = 4096
    dt = 0.1 / (nx - 2)
    steps = int(round(0.2 / dt))
    cfg = sw.make_config(2, 8, alg=sw.ALG_SWEPT, nx=nx, tpb=256, dt=dt, time_mode=sw.TIME_STEPS, n_steps=steps)
    fin, res, _ = solver.run(cfg)
    q = fin.reshape(-1, 3)
    ex = exact.sod(exact.sod_cell_centres(nx), steps * dt)
    err = float(np.mean(np.abs(q[1:-1, 0] - ex["density"])))
    assert err < 0.001, err


@pytest.mark.parametrize("prec", [8, 4])
def test_euler_2_22_swept_equals_oracle(sw, solver, oracle, prec):
    """Euler Sod at config 3's size (nx=2^22, tpb=512, dt/dx=0.1): the swept run
    over 256 steps (one up-triangle, diamonds, a down-triangle and classic
    remainder steps) equals the oracle's classic scheme bit for bit, the oracle
    on every host thread."""
    nx, tpb, steps = 1 << 22, 512, 256 + 37
    dt = 0.1 / (nx - 2)
    cfg = sw.make_config(2, prec, alg=sw.ALG_SWEPT, nx=nx, tpb=tpb, dt=dt, time_mode=sw.TIME_STEPS, n_steps=steps)
    ic = oracle.reference_ic(oracle.EULER, prec, nx)
    want = oracle.classic(oracle.reference_consts(oracle.EULER, prec, nx, dt), ic, steps,
                          threads=oracle.openmp_threads())
    got, res, _ = solver.run(cfg, ic)
    assert res.n_steps == steps
    assert np.isfinite(got).all()
    np.testing.assert_array_equal(got, want)
