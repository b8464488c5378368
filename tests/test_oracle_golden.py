"""The oracle against the reference: golden vectors made by the reference's own
code (tests/golden/make_golden.py), the reference's KS golden run, and the
analytic solutions its accuracy tests use.  CPU only."""
import math

import numpy as np
import pytest

from oracle import exact

CASES = [(p, q) for p in ("heat", "ks", "euler") for q in (64, 32)]
PID = {"heat": 0, "ks": 1, "euler": 2}


@pytest.mark.parametrize("name,bits", CASES)
def test_initial_condition_is_reference(oracle, golden, name, bits):
    """or_reference_ic == the reference's initFun / Sod IC, bit for bit."""
    key = "%s_f%d" % (name, bits)
    ref = golden["ref"][key + "_ic"]
    nx = int(golden["ref"][key + "_meta"][0])
    mine = oracle.reference_ic(PID[name], bits // 8, nx)
    assert mine.dtype == ref.dtype
    np.testing.assert_array_equal(mine, ref)


@pytest.mark.parametrize("name,bits", CASES)
def test_classic_is_reference_bit_exact(oracle, golden, name, bits):
    """The oracle's classic loop == the reference's own stencil functions
    (execFunc / stutterStep+finalStep / eulerStutterStep+eulerFinalStep), bit for bit."""
    key = "%s_f%d" % (name, bits)
    nx, dt, nsteps = golden["ref"][key + "_meta"]
    c = oracle.reference_consts(PID[name], bits // 8, int(nx), dt)
    out = oracle.classic(c, golden["ref"][key + "_ic"], int(nsteps))
    np.testing.assert_array_equal(out, golden["ref"][key + "_final"])


@pytest.mark.parametrize("bits", [64, 32])
def test_ks_divide_is_reference_bit_exact(oracle, golden, bits):
    """The oracle's divide form == the reference's DIVISE-build stencil functions
    (KS1D_SweptShared.cu:111-132) at dx = 0.3, bit for bit; and its reciprocal
    form == the reference's default build there, which rounds differently."""
    g = golden["ks_divide"]
    nx, dt, dx, nsteps = g["meta"]
    prec = bits // 8
    for divide, key in ((True, "divide"), (False, "multiply")):
        c = oracle.ks_consts(prec, int(nx), dt, dx=dx, divide=divide)
        out = oracle.classic(c, g["f%d_ic" % bits], int(nsteps))
        np.testing.assert_array_equal(out, g["f%d_%s" % (bits, key)])
    assert not np.array_equal(g["f%d_divide" % bits], g["f%d_multiply" % bits])


@pytest.mark.parametrize("bits", [64, 32])
def test_euler_pressure_is_reference(oracle, golden, bits):
    """The .dat Pressure row: oracle pressure() == the reference's pressure()."""
    key = "euler_f%d" % bits
    nx, dt, _ = golden["ref"][key + "_meta"]
    c = oracle.reference_consts(2, bits // 8, int(nx), dt)
    fin = golden["ref"][key + "_final"]
    np.testing.assert_array_equal(oracle.euler_pressure(c, fin), golden["ref"][key + "_pressure"])


def test_openmp_classic_equals_serial(oracle):
    """The CPU baseline (OpenMP) computes exactly what the serial oracle does."""
    for p in (0, 1, 2):
        c = oracle.reference_consts(p, 8, 8192, {0: 0.004, 1: 0.005, 2: 0.1 / 8190}[p])
        ic = oracle.reference_ic(p, 8, 8192)
        np.testing.assert_array_equal(oracle.classic(c, ic, 37), oracle.classic(c, ic, 37, threads=4))


@pytest.mark.parametrize("problem", [0, 1, 2])
@pytest.mark.parametrize("tpb", [32, 64, 128])
@pytest.mark.parametrize("bc", [None, "periodic"])
def test_swept_model_equals_classic(oracle, problem, tpb, bc):
    """CPU model of the GPU swept decomposition == classic, bit for bit, for
    odd and even diamond counts (down-triangle in both phases)."""
    if bc == "periodic" and problem != 0:
        pytest.skip("periodic override only differs from the default for Heat")
    nx = 8 * tpb
    dt = {0: 0.004, 1: 0.005, 2: 0.1 / (nx - 2)}[problem]
    c = oracle.reference_consts(problem, 8, nx, dt)
    if bc == "periodic":
        c.bc = oracle.BC_PERIODIC
    rng = np.random.default_rng(tpb + problem)
    ic = oracle.reference_ic(problem, 8, nx)
    if problem != 2:
        ic = ic + 0.01 * rng.standard_normal(ic.size)
    for nd in (0, 1, 2, 5):
        s, n = oracle.swept(c, ic, tpb, nd)
        np.testing.assert_array_equal(s, oracle.classic(c, ic, n))


def test_swept_model_rejects_bad_tiles(oracle):
    c = oracle.reference_consts(1, 8, 256, 0.005)
    with pytest.raises(ValueError):
        oracle.swept(c, oracle.reference_ic(1, 8, 256), 12, 1)  # not a multiple of 4R
    with pytest.raises(ValueError):
        oracle.swept(c, oracle.reference_ic(1, 8, 256), 96, 1)  # does not divide nx


def test_ks_official_golden(oracle, golden):
    """KS against the reference's golden run (Testing/KSDouble_Official.txt:
    FP64 swept, dt = 1e-7).  The IC row is the oracle's IC to the file's 10
    digits; the oracle's classic run at dt = 1e-5 reaches t = 6 within 1e-7
    of it (max abs; the values are O(1))."""
    g = golden["ks"]
    lx, nx, dx = g["header"]
    nx = int(nx)
    assert (lx, dx) == (512.0, 0.5)
    ic = oracle.reference_ic(1, 8, nx)
    np.testing.assert_allclose(ic, g["velocity"][0], rtol=0, atol=5e-10 * 2)
    assert list(g["times"]) == [0.0, 6.0, 12.0, 18.0, 20.0]
    dt = 1e-5
    c = oracle.reference_consts(1, 8, nx, dt)
    u = oracle.classic(c, ic, int(round(6.0 / dt)), threads=4)
    err = float(np.abs(u - g["velocity"][1]).max())
    assert err < 1e-7, err


def test_heat_series_matches_classic(oracle):
    """testProcedure's heat_exact series vs the classic scheme (nx=1024, dt=1e-4,
    t = 1): RMSE under 0.05 (the series uses L = nx*dx while the program's rod is
    (nx-1)*dx long -- a known offset of the reference's own test)."""
    nx, dt, t = 1024, 1e-4, 1.0
    c = oracle.reference_consts(0, 8, nx, dt)
    u = oracle.classic(c, oracle.reference_ic(0, 8, nx), int(round(t / dt)), threads=4)
    rmse = math.sqrt(float(np.mean((u - exact.heat_series(t, nx)) ** 2)))
    assert rmse < 0.05, rmse


def test_heat_periodic_mode_exact(oracle):
    """Periodic FTCS with a sine IC decays by exactly (1 - 4 Fo sin^2(pi/nx))^n."""
    nx, fo = 4096, 0.1
    c = oracle.reference_consts(0, 8, nx, 1e-3)
    c.bc = oracle.BC_PERIODIC
    c.fourier, c.fourier_two = fo, 1 - 2 * fo
    x = np.arange(nx)
    ic = 50 + 100 * np.sin(2 * np.pi * x / nx)
    u = oracle.classic(c, ic, 2000, threads=4)
    want = exact.heat_periodic_mode(2000, nx, fo)
    assert np.abs(u - want).max() < 1e-10


def test_sod_exact_star_state():
    """Exact Riemann solver: Sod star state (Toro, Test 1: p* = 0.30313, u* = 0.92745)."""
    p, u = exact.sod_star()
    assert abs(p - 0.30313) < 1e-5 and abs(u - 0.92745) < 1e-5


def test_sod_classic_converges(oracle):
    """Classic Euler vs the exact Sod solution at t = 0.2: density L1 error
    falls with resolution and is below 0.01 at 1024 interior cells."""
    errs = []
    for nx in (258, 1026):
        dt = 0.1 / (nx - 2)
        c = oracle.reference_consts(2, 8, nx, dt)
        q = oracle.classic(c, oracle.reference_ic(2, 8, nx), int(round(0.2 / dt)), threads=4).reshape(-1, 3)
        x = exact.sod_cell_centres(nx)
        ex = exact.sod(x, 0.2)
        errs.append(float(np.mean(np.abs(q[1:-1, 0] - ex["density"]))))
    assert errs[1] < errs[0] and errs[1] < 0.01, errs


@pytest.mark.parametrize("problem", [0, 1, 2])
def test_fp32_close_to_fp64(oracle, problem):
    """FP32 runs track FP64 within 1e-5 relative on smooth short runs."""
    nx = 1024
    dt = {0: 0.004, 1: 0.005, 2: 0.1 / (nx - 2)}[problem]
    u64 = oracle.classic(oracle.reference_consts(problem, 8, nx, dt), oracle.reference_ic(problem, 8, nx), 50)
    u32 = oracle.classic(oracle.reference_consts(problem, 4, nx, dt), oracle.reference_ic(problem, 4, nx), 50)
    scale = np.abs(u64).max()
    assert np.abs(u32.astype(np.float64) - u64).max() / scale < 1e-5


def test_closure_oracle_gradient_is_exact():
    """The closure oracle's analytic gradient equals central differences of its
    loss (BF16 rounding switched off, since it makes the loss piecewise constant)."""
    from oracle import closure as ocl
    th = ocl.init(1).astype(np.float64)
    rng = np.random.default_rng(3)
    th[5344:5505] = rng.standard_normal(161) * 0.1
    th[5505] = 0.7
    u = rng.standard_normal((2, 64))
    tgt = rng.standard_normal((2, 64)) * 0.1
    saved = ocl.bf16
    ocl.bf16 = lambda x: np.asarray(x, dtype=np.float64)
    try:
        _, g = ocl.loss_and_grad(th, u, tgt)
        assert g[5505] == 0.0
        for i in (0, 40, 100, 170, 200, 3000, 5300, 5320, 5400, 5504):
            e = np.zeros_like(th)
            e[i] = 1e-6
            fd = (ocl.loss_and_grad(th + e, u, tgt)[0] - ocl.loss_and_grad(th - e, u, tgt)[0]) / 2e-6
            assert abs(g[i] - fd) <= 1e-6 * max(1.0, abs(fd)), (i, g[i], fd)
    finally:
        ocl.bf16 = saved


def test_closure_oracle_bf16_rounding():
    from oracle import closure as ocl
    x = np.array([1.0, 1.00390625, 1.005859375, 3.14159, -2.5e-3, 0.0], dtype=np.float32)
    r = ocl.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0      # halfway: ties to even
    assert r[2] == 1.0078125                # above halfway rounds up
    assert abs(r[3] - 3.140625) < 1e-12
    assert (ocl.bf16(r) == r).all()          # idempotent
