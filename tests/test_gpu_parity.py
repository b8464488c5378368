"""GPU parity: the CUDA paths (classic, swept, persistent variant) through the C
ABI against the CPU oracle on the same inputs.  The bar is bit-identity: every
path computes each (cell, sub-step) once with the reference's arithmetic, so
the FP64 and FP32 results must equal the oracle's exactly (which is stricter
than the 1e-12 / 1e-5 relative tolerances the spec allows)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HEAT, KS, EULER = 0, 1, 2
CLASSIC, SWEPT, VARIANT = 0, 1, 2
TIME_STEPS = 1


def _case(oracle, problem, prec, nx, dt, bc=None, **over):
    c = oracle.reference_consts(problem, prec, nx, dt)
    if bc is not None:
        c.bc = bc
    for k, v in over.items():
        setattr(c, k, v)
    return c


def _ic(oracle, problem, prec, nx, kind="reference", seed=0):
    if kind == "reference":
        return oracle.reference_ic(problem, prec, nx)
    rng = np.random.default_rng(seed)
    dt = np.float64 if prec == 8 else np.float32
    if problem == EULER:
        u = oracle.reference_ic(problem, prec, nx).reshape(-1, 3).astype(np.float64)
        rho = 0.5 + rng.random(nx)
        rho[0], rho[-1] = u[0, 0], u[-1, 0]
        mom = 0.1 * rng.standard_normal(nx)
        mom[0] = mom[-1] = 0
        p = 0.2 + rng.random(nx)
        E = p / 0.4 + 0.5 * mom ** 2 / rho
        E[0], E[-1] = u[0, 2], u[-1, 2]
        return np.stack([rho, mom, E], 1).astype(dt).ravel()
    x = np.arange(nx)
    return (50 + 40 * np.sin(2 * np.pi * x / nx) + rng.standard_normal(nx)).astype(dt) if problem == HEAT else \
        (np.cos(2 * np.pi * 3 * x / nx) + 0.1 * rng.standard_normal(nx)).astype(dt)


def _gpu(sw, solver, problem, prec, alg, nx, tpb, dt, nsteps, ic, bc=0):
    cfg = sw.make_config(problem, prec, alg=alg, nx=nx, tpb=tpb, dt=dt, time_mode=TIME_STEPS, n_steps=nsteps, bc=bc)
    fin, res, _ = solver.run(cfg, ic)
    assert res.n_steps == nsteps
    return fin, res


def _assert_identical(a, b, what):
    assert a.dtype == b.dtype
    if not np.array_equal(a, b):
        d = np.abs(a.astype(np.float64) - b.astype(np.float64))
        i = int(np.argmax(d))
        raise AssertionError("%s: %d of %d cells differ, max |diff| %.3e at %d (%r vs %r)" % (
            what, int((d > 0).sum()), a.size, d[i], i, a.ravel()[i], b.ravel()[i]))


PROBLEM_DT = {HEAT: 0.004, KS: 0.005, EULER: 0.1 / 254}


@pytest.mark.parametrize("prec", [8, 4])
@pytest.mark.parametrize("problem", [HEAT, KS, EULER])
@pytest.mark.parametrize("alg", [CLASSIC, SWEPT, VARIANT])
def test_reference_ic_bit_exact(sw, solver, oracle, problem, prec, alg):
    """Reference IC and constants, 256 cells, tile 64: every path == oracle."""
    nx, tpb, dt = 256, 64, PROBLEM_DT[problem]
    c = _case(oracle, problem, prec, nx, dt)
    ic = _ic(oracle, problem, prec, nx)
    q = tpb // (2 * oracle.RADIUS[problem] * oracle.SUBSTEPS[problem])
    for nsteps in (0, 1, q, 2 * q, 3 * q + 1, 7 * q):
        want = oracle.classic(c, ic, nsteps)
        got, _ = _gpu(sw, solver, problem, prec, alg, nx, tpb, dt, nsteps, ic)
        _assert_identical(got, want, "problem %d prec %d alg %d steps %d" % (problem, prec, alg, nsteps))


@pytest.mark.parametrize("tpb", [32, 64, 128, 256, 512, 1024])
@pytest.mark.parametrize("problem", [HEAT, KS, EULER])
def test_tile_widths(sw, solver, oracle, problem, tpb):
    """Every tile width, random ICs, FP64, swept and variant, several diamond counts."""
    nx = max(4 * tpb, 1024)
    dt = PROBLEM_DT[problem] if problem != EULER else 0.1 / (nx - 2)
    c = _case(oracle, problem, 8, nx, dt)
    ic = _ic(oracle, problem, 8, nx, kind="random", seed=tpb)
    q = tpb // (2 * oracle.RADIUS[problem] * oracle.SUBSTEPS[problem])
    for nsteps in (q, 2 * q + 3, 5 * q):
        want = oracle.classic(c, ic, nsteps)
        for alg in (SWEPT, VARIANT):
            if problem == KS and alg == VARIANT and tpb != 32:
                continue  # KS variant always uses 32-cell nodes; covered below
            got, _ = _gpu(sw, solver, problem, 8, alg, nx, tpb, dt, nsteps, ic)
            _assert_identical(got, want, "problem %d tpb %d alg %d steps %d" % (problem, tpb, alg, nsteps))


@pytest.mark.parametrize("prec", [8, 4])
@pytest.mark.parametrize("problem", [HEAT, KS, EULER])
def test_threads_per_block(sw, solver, oracle, problem, prec):
    """Any threads per swept block gives the same bits: 4 contiguous cells per
    thread (tpb / 4), a strided walk (tpb / 2, 32), one per cell, and requests
    out of range (33, 2 * tpb, 4096) that fall back to the default."""
    nx, tpb = 2048, 256
    dt = PROBLEM_DT[problem] if problem != EULER else 0.1 / (nx - 2)
    c = _case(oracle, problem, prec, nx, dt)
    ic = _ic(oracle, problem, prec, nx, kind="random", seed=17)
    q = tpb // (2 * oracle.RADIUS[problem] * oracle.SUBSTEPS[problem])
    nsteps = 3 * q + 1
    want = oracle.classic(c, ic, nsteps)
    for alg in (SWEPT, VARIANT):
        for th in (0, 32, 64, 128, 256, 33, 512, 4096):
            cfg = sw.make_config(problem, prec, alg=alg, nx=nx, tpb=tpb, dt=dt, time_mode=TIME_STEPS, n_steps=nsteps)
            cfg.threads = th
            got, _, _ = solver.run(cfg, ic)
            _assert_identical(got, want, "problem %d prec %d alg %d threads %d" % (problem, prec, alg, th))


@pytest.mark.parametrize("problem, prec, tpb, bc", [(KS, 8, 64, 0), (KS, 4, 64, 0), (HEAT, 8, 32, 0),
                                                    (HEAT, 8, 64, 2), (HEAT, 4, 32, 0), (KS, 8, 512, 0),
                                                    (KS, 4, 256, 0), (HEAT, 4, 128, 0), (HEAT, 4, 128, 2)])
def test_grouped_tiles(sw, solver, oracle, problem, prec, tpb, bc):
    """Domains of >= 1024 tiles with the default thread shape run several tiles
    per block (KS four, two at tpb 512; Heat two), their live cells packed
    together at every level: one cell per thread, and 4 cells per thread in
    FP32 from tpb 128 (KS from 256; its 128-cell tiles take the warp kernel)."""
    nx = 1024 * tpb
    dt = PROBLEM_DT[problem]
    c = _case(oracle, problem, prec, nx, dt, bc=oracle.BC_PERIODIC if bc == 2 else None)
    ic = _ic(oracle, problem, prec, nx, kind="random", seed=21)
    q = tpb // (2 * oracle.RADIUS[problem] * oracle.SUBSTEPS[problem])
    for nsteps in (q, 3 * q + 1):
        want = oracle.classic(c, ic, nsteps)
        got, _ = _gpu(sw, solver, problem, prec, SWEPT, nx, tpb, dt, nsteps, ic, bc=bc)
        _assert_identical(got, want, "problem %d prec %d tpb %d bc %d steps %d" % (problem, prec, tpb, bc, nsteps))


@pytest.mark.parametrize("prec", [8, 4])
def test_heat_periodic(sw, solver, oracle, prec):
    """Heat on a periodic domain (the benchmark's boundary), all paths."""
    nx, tpb, dt = 1024, 128, 0.004
    c = _case(oracle, HEAT, prec, nx, dt, bc=oracle.BC_PERIODIC)
    ic = _ic(oracle, HEAT, prec, nx, kind="random", seed=3)
    for alg in (CLASSIC, SWEPT, VARIANT):
        for nsteps in (64, 128, 640, 701):
            want = oracle.classic(c, ic, nsteps)
            got, _ = _gpu(sw, solver, HEAT, prec, alg, nx, tpb, dt, nsteps, ic, bc=2)
            _assert_identical(got, want, "periodic heat alg %d steps %d" % (alg, nsteps))


@pytest.mark.parametrize("problem", [HEAT, KS, EULER])
def test_single_tile_domain(sw, solver, oracle, problem):
    """nx == tpb: the shifted tile wraps onto the same tile's halves."""
    nx = tpb = 64
    dt = PROBLEM_DT[problem] if problem != EULER else 0.1 / 62
    c = _case(oracle, problem, 8, nx, dt)
    ic = _ic(oracle, problem, 8, nx, kind="random", seed=9)
    for nsteps in (8, 32, 96):
        want = oracle.classic(c, ic, nsteps)
        for alg in (SWEPT, VARIANT):
            got, _ = _gpu(sw, solver, problem, 8, alg, nx, tpb, dt, nsteps, ic)
            _assert_identical(got, want, "single tile problem %d alg %d" % (problem, alg))


def test_ks_variant_32_cell_nodes(sw, solver, oracle):
    """KS alg 2 runs 32-cell nodes whatever tpb says (the reference's register path)."""
    nx, dt = 2048, 0.005
    c = _case(oracle, KS, 8, nx, dt)
    ic = _ic(oracle, KS, 8, nx)
    want = oracle.classic(c, ic, 40)
    got, res = _gpu(sw, solver, KS, 8, VARIANT, nx, 256, dt, 40, ic)
    assert res.tile == 32
    _assert_identical(got, want, "ks variant")


def _nonnormal_ic(problem, nx, seed):
    """A state whose products leave the integer pipe's range: subnormal cells
    (1e-310), zeros, cells whose KS squares are subnormal (1e-160) or overflow
    (1e155), and for Heat three neighbouring cells of 1.7e308 (the middle
    one's neighbours' sum overflows), among ordinary values."""
    rng = np.random.default_rng(seed)
    x = np.arange(nx)
    if problem == HEAT:
        u = 50 + 40 * np.sin(2 * np.pi * x / nx) + rng.standard_normal(nx)
        specials = ((1e-310, 24), (-3e-312, 8), (0.0, 16), (-0.0, 8), (1.7e308, 1))
    else:
        u = np.cos(2 * np.pi * 3 * x / nx) + 0.1 * rng.standard_normal(nx)
        specials = ((1e-310, 24), (-3e-312, 8), (1e-160, 24), (0.0, 16), (-0.0, 8), (1e155, 1))
    for value, count in specials:
        u[rng.choice(nx, count, replace=False)] = value
    if problem == HEAT:  # a cell whose neighbours' sum overflows
        k = int(np.argmax(u))
        u[(k + 1) % nx] = u[(k + 2) % nx] = u[k]
    return u


def _assert_same_or_both_nan(a, b, what):
    """Bit-identical where finite or infinite; NaN where the other is NaN (the
    payload and sign of a NaN differ between the CPU and the GPU)."""
    na, nb = np.isnan(a), np.isnan(b)
    assert np.array_equal(na, nb), "%s: NaN at different cells" % what
    assert na.sum() < a.size // 4, "%s: too many NaN cells for a meaningful check" % what
    _assert_identical(np.where(na, 0.0, a), np.where(nb, 0.0, b), what)


@pytest.mark.parametrize("problem, alg, nx, tpb, bc", [
    (KS, CLASSIC, 4096, 64, 0), (KS, SWEPT, 4096, 64, 0), (KS, SWEPT, 16384, 1024, 0), (KS, SWEPT, 65536, 64, 0),
    (KS, SWEPT, 262144, 256, 0), (KS, VARIANT, 4096, 64, 0),
    (HEAT, CLASSIC, 4096, 64, 0), (HEAT, CLASSIC, 4096, 64, 2), (HEAT, SWEPT, 4096, 64, 0), (HEAT, SWEPT, 4096, 64, 2),
    (HEAT, SWEPT, 16384, 1024, 0), (HEAT, SWEPT, 32768, 32, 0), (HEAT, SWEPT, 65536, 64, 2), (HEAT, VARIANT, 4096, 64, 0),
    (HEAT, VARIANT, 4096, 128, 2),
    # 512 tiles: enough for the integer products on the one-tile-per-block and persistent kernels
    (KS, SWEPT, 1 << 19, 1024, 0), (KS, VARIANT, 32768, 64, 0), (HEAT, SWEPT, 1 << 19, 1024, 2),
    (HEAT, VARIANT, 32768, 64, 0)])
def test_fp64_values_outside_the_integer_products(sw, solver, oracle, problem, alg, nx, tpb, bc):
    """FP64 Heat and KS form their general products on the integer pipe and
    compute a cell again on the FP64 pipe where an operand or a product is
    outside that path's range; domains of fewer tiles than two per SM keep
    every product on the FP64 pipe.  With such values in the state every path
    (classic, one tile per block, two cells per thread at tpb 1024, grouped
    tiles, the persistent variant and KS's 32-cell nodes, on few and on many
    tiles; insulated and periodic Heat) still gives the oracle's bits."""
    dt = PROBLEM_DT[problem]
    c = _case(oracle, problem, 8, nx, dt, bc=oracle.BC_PERIODIC if bc == 2 else None)
    ic = _nonnormal_ic(problem, nx, seed=nx + tpb + bc)
    q = tpb // (2 * oracle.RADIUS[problem] * oracle.SUBSTEPS[problem])
    for nsteps in (q, 2 * q + 3):
        want = oracle.classic(c, ic, nsteps)
        got, _ = _gpu(sw, solver, problem, 8, alg, nx, tpb, dt, nsteps, ic, bc=bc)
        _assert_same_or_both_nan(got, want, "problem %d alg %d nx %d tpb %d bc %d steps %d" % (
            problem, alg, nx, tpb, bc, nsteps))


def _euler_special_ic(oracle, nx, seed):
    """A Sod tube with edge-case states in places: momenta of +-1e-160 (their
    squares underflow to subnormals), +-1e-310 (subnormal), zeros of both
    signs, and density and energy jumps of one rounding unit."""
    rng = np.random.default_rng(seed)
    u = oracle.reference_ic(EULER, 8, nx).reshape(-1, 3).copy()
    inner = np.arange(2, nx - 2)
    for value, count in ((1e-160, 12), (-1e-160, 12), (1e-310, 6), (-3e-312, 6), (-0.0, 24)):
        u[rng.choice(inner, count, replace=False), 1] = value
    k = rng.choice(inner, 12, replace=False)
    u[k, 0] *= 1 + 1e-15
    u[k, 2] *= 1 - 1e-15
    return u.ravel()


@pytest.mark.parametrize("alg, nx, tpb", [(CLASSIC, 4096, 256), (SWEPT, 4096, 256), (VARIANT, 4096, 256),
                                          (SWEPT, 1 << 16, 512), (VARIANT, 1 << 15, 256), (CLASSIC, 1 << 16, 512)])
def test_euler_edge_case_states(sw, solver, oracle, alg, nx, tpb):
    """Subnormal and underflowing momenta, signed zeros and one-ulp jumps in
    a Sod tube: every FP64 Euler path (classic, swept on few and many tiles,
    the persistent variant) gives the oracle's bits."""
    dt = 0.1 / (nx - 2)
    c = _case(oracle, EULER, 8, nx, dt)
    ic = _euler_special_ic(oracle, nx, seed=nx + tpb + alg)
    q = tpb // (2 * oracle.RADIUS[EULER] * oracle.SUBSTEPS[EULER])
    for nsteps in (q, 2 * q + 3):
        want = oracle.classic(c, ic, nsteps)
        got, _ = _gpu(sw, solver, EULER, 8, alg, nx, tpb, dt, nsteps, ic)
        _assert_same_or_both_nan(got, want, "euler alg %d nx %d tpb %d steps %d" % (alg, nx, tpb, nsteps))


@pytest.mark.parametrize("problem", [HEAT, KS, EULER])
def test_reference_time_mode_snapshots(sw, solver, oracle, problem):
    """SW_TIME_REFERENCE: snapshots at the reference's output times hold the
    oracle state after the matching step counts."""
    nx, tpb = 512, 64
    dt = {HEAT: 0.004, KS: 0.005, EULER: 0.1 / 510}[problem]
    q = tpb // (2 * oracle.RADIUS[problem] * oracle.SUBSTEPS[problem])
    tf = 60 * q * dt
    freq = 17 * q * dt
    c = _case(oracle, problem, 8, nx, dt)
    ic = _ic(oracle, problem, 8, nx)
    finals = {}
    for alg in (CLASSIC, SWEPT, VARIANT):
        cfg = sw.make_config(problem, 8, alg=alg, nx=nx, tpb=tpb, dt=dt, tf=tf, freq=freq)
        fin, res, snaps = solver.run(cfg, ic)
        assert len(snaps) >= 2
        # every swept snapshot time is a whole number of half-cycles; the state matches the oracle there
        for t, state in snaps:
            n = int(round(t / dt))
            if alg == CLASSIC and problem == HEAT:
                continue  # classic Heat advances t_eq one extra pass per snapshot (checked below)
            _assert_identical(state, oracle.classic(c, ic, n), "snapshot alg %d t %.6f" % (alg, t))
        _assert_identical(fin, oracle.classic(c, ic, res.n_steps), "final alg %d" % alg)
        finals[alg] = (res.t_final, res.n_steps)
    assert finals[SWEPT] == finals[VARIANT] or problem == KS


def test_run_device_torch(sw, solver, oracle):
    """sw_run_device on a torch CUDA tensor (device layout), in place."""
    torch = pytest.importorskip("torch")
    nx, tpb, dt = 4096, 256, 0.005
    c = _case(oracle, KS, 8, nx, dt)
    ic = _ic(oracle, KS, 8, nx)
    t = torch.from_numpy(ic.copy()).cuda()
    cfg = sw.make_config(KS, 8, alg=SWEPT, nx=nx, tpb=tpb, dt=dt, time_mode=TIME_STEPS, n_steps=320)
    res = solver.run_device(cfg, t.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert res.n_steps == 320
    _assert_identical(t.cpu().numpy(), oracle.classic(c, ic, 320), "run_device")


def test_euler_device_layout(sw, solver, oracle):
    """Euler device layout is (rho, rho u, E, pad) per cell."""
    torch = pytest.importorskip("torch")
    nx, tpb, dt = 1024, 128, 0.1 / 1022
    c = _case(oracle, EULER, 8, nx, dt)
    ic = _ic(oracle, EULER, 8, nx)
    dev = np.zeros((nx, 4))
    dev[:, :3] = ic.reshape(-1, 3)
    t = torch.from_numpy(dev).cuda()
    cfg = sw.make_config(EULER, 8, alg=SWEPT, nx=nx, tpb=tpb, dt=dt, time_mode=TIME_STEPS, n_steps=96)
    solver.run_device(cfg, t.data_ptr())
    out = t.cpu().numpy()
    _assert_identical(np.ascontiguousarray(out[:, :3]).ravel(), oracle.classic(c, ic, 96), "euler device")
    assert (out[:, 3] == 0).all()


def test_bounded_wait_reports_timeout(sw, solver, oracle):
    """The persistent kernels' wait, on a flag nothing sets, gives up after its
    limit and reports SW_ERR_TIMEOUT through the status word; the context then
    runs a solve normally."""
    rc, ms = solver.wait_probe(50_000_000)  # 50 ms
    assert rc == -7, rc
    assert 40.0 < ms < 2000.0, ms
    nx, dt = 256, 0.005
    c = _case(oracle, KS, 8, nx, dt)
    ic = _ic(oracle, KS, 8, nx)
    got, _ = _gpu(sw, solver, KS, 8, VARIANT, nx, 64, dt, 40, ic)
    _assert_identical(got, oracle.classic(c, ic, 40), "after the timeout")
    assert solver.wait_probe(10)[0] == -1  # limit out of range: SW_ERR_ARG, nothing launched


@pytest.mark.parametrize("nx", [128, 256, 4096])
def test_ks_fp32_warp_tiles(sw, solver, oracle, nx):
    """FP32 KS swept at tile 128 runs each tile in one warp's registers: bit for
    bit the oracle, for a single-tile domain (both halves wrap onto the same
    tile), two tiles and many, over several diamond counts and remainders."""
    dt = PROBLEM_DT[KS]
    c = _case(oracle, KS, 4, nx, dt)
    ic = _ic(oracle, KS, 4, nx, kind="random", seed=nx)
    for nsteps in (16, 32, 33, 160, 321):
        want = oracle.classic(c, ic, nsteps)
        got, _ = _gpu(sw, solver, KS, 4, SWEPT, nx, 128, dt, nsteps, ic)
        _assert_identical(got, want, "fp32 ks warp tiles nx %d steps %d" % (nx, nsteps))
