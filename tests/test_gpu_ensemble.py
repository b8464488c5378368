"""Ensembles on the GPU: many independent domains of uneven length in one
launch per pass (swept), one persistent launch (variant) or per-step launches
(classic), through sw_run_batch / sw_run_batch_device; every domain must
equal the oracle run on that domain alone, bit for bit."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ens = importlib.import_module("1dsweptcuda_gb300.ensemble")


def _oracle_each(oracle, problem, prec, nx, state, dt, steps, comps=1, **over):
    outs = []
    for part, n in zip(ens.split(state, nx, comps), nx):
        c = oracle.reference_consts(problem, prec, int(n), dt)
        for k, v in over.items():
            setattr(c, k, v)
        outs.append(oracle.classic(c, part, steps))
    return ens.concat(outs)


@pytest.mark.parametrize("prec", [8, 4])
@pytest.mark.parametrize("alg", [0, 1, 2])
def test_ks_ensemble_bit_exact(sw, solver, oracle, prec, alg):
    nx, ic = ens.make_ensemble(n_domains=24, lo=6, hi=11, seed=5, dtype=np.float64 if prec == 8 else np.float32)
    dt, steps = 0.005, 52   # 6 diamonds of 8 steps at tile 64, then 4 classic steps
    cfg = sw.make_config(1, prec, alg=alg, tpb=64, dt=dt, time_mode=sw.TIME_STEPS, n_steps=steps)
    out, res = solver.run_batch(cfg, nx, ic)
    assert res.n_steps == steps
    want = _oracle_each(oracle, 1, prec, nx, ic, dt, steps)
    np.testing.assert_array_equal(out, want)


@pytest.mark.parametrize("prec", [8, 4])
def test_ensembles_of_grouped_tiles(sw, solver, oracle, prec):
    """Every domain a multiple of four tiles (KS) or two (Heat), one cell per
    thread, at least 1024 tiles in all: the swept passes run G tiles of one
    domain per block, as the single-domain kernel groups them (FP64 KS with
    bulk-copied slots).  Every domain still equals the oracle run on it alone."""
    dt = np.float64 if prec == 8 else np.float32
    nx, ic = ens.make_ensemble(n_domains=96, lo=8, hi=11, seed=7, dtype=dt)
    assert nx.sum() // 64 >= 1024
    cfg = sw.make_config(1, prec, alg=1, tpb=64, dt=0.005, time_mode=sw.TIME_STEPS, n_steps=52)
    out, res = solver.run_batch(cfg, nx, ic)
    assert res.n_steps == 52
    np.testing.assert_array_equal(out, _oracle_each(oracle, 1, prec, nx, ic, 0.005, 52))
    rng = np.random.default_rng(3)
    nx = np.tile(np.array([256, 128, 512, 128, 1024], dtype=np.int64), 40)
    ic = (rng.standard_normal(int(nx.sum())) + 10.0).astype(dt)
    cfg = sw.make_config(0, prec, alg=1, tpb=64, dt=0.004, bc=sw.BC_PERIODIC, time_mode=sw.TIME_STEPS, n_steps=100)
    out, _ = solver.run_batch(cfg, nx, ic)
    np.testing.assert_array_equal(out, _oracle_each(oracle, 0, prec, nx, ic, 0.004, 100, bc=oracle.BC_PERIODIC))
    cfg = sw.make_config(0, prec, alg=1, tpb=64, dt=0.004, time_mode=sw.TIME_STEPS, n_steps=100)  # insulated ends
    out, _ = solver.run_batch(cfg, nx, ic)
    np.testing.assert_array_equal(out, _oracle_each(oracle, 0, prec, nx, ic, 0.004, 100))


def test_heat_periodic_and_euler_ensembles(sw, solver, oracle):
    rng = np.random.default_rng(1)
    nx = np.array([128, 512, 256, 1024, 128], dtype=np.int64)
    ic = rng.standard_normal(int(nx.sum())) + 10.0
    cfg = sw.make_config(0, 8, alg=1, tpb=64, dt=0.004, bc=sw.BC_PERIODIC, time_mode=sw.TIME_STEPS, n_steps=100)
    out, _ = solver.run_batch(cfg, nx, ic)
    np.testing.assert_array_equal(out, _oracle_each(oracle, 0, 8, nx, ic, 0.004, 100, bc=oracle.BC_PERIODIC))
    # Euler: Sod tube in every domain, one dx for all (set explicitly)
    nx = np.array([256, 1024, 512], dtype=np.int64)
    parts = [oracle.reference_ic(2, 8, int(n)) for n in nx]
    ic = ens.concat(parts)
    dx, dt = 1.0 / 254, 0.1 / 254
    for alg in (0, 1, 2):
        cfg = sw.make_config(2, 8, alg=alg, tpb=64, dt=dt, dx=dx, time_mode=sw.TIME_STEPS, n_steps=40)
        out, _ = solver.run_batch(cfg, nx, ic)
        np.testing.assert_array_equal(out, _oracle_each(oracle, 2, 8, nx, ic, dt, 40, comps=3, dt_dx=dt / dx))


def test_graph_replay_and_device_entry(sw, solver, oracle):
    """The second identical call replays the captured graph; device entry point in place."""
    torch = pytest.importorskip("torch")
    nx, ic = ens.make_ensemble(n_domains=40, lo=7, hi=12, seed=9)
    cfg = sw.make_config(1, 8, alg=2, tpb=128, dt=0.005, time_mode=sw.TIME_STEPS, n_steps=64)
    want = _oracle_each(oracle, 1, 8, nx, ic, 0.005, 64)
    for _ in range(3):
        t = torch.from_numpy(ic.copy()).cuda()
        res = solver.run_batch_device(cfg, nx, t.data_ptr())
        np.testing.assert_array_equal(t.cpu().numpy(), want)
    assert res.launches == 1  # one persistent cooperative launch


def test_autotuner(sw, solver, oracle):
    nx, ic = ens.make_ensemble(n_domains=64, lo=10, hi=13, seed=2)
    cfg = sw.make_config(1, 8, alg=1, tpb=0, dt=0.005, time_mode=sw.TIME_STEPS, n_steps=96)
    t = solver.tune(cfg, nx)
    cands = t.candidates()
    assert t.n_candidates >= 6
    assert (t.tile, t.threads) in [(a, b) for a, b, _ in cands]
    assert t.cell_updates_per_s == max(r for _, _, r in cands)
    assert all(nx % t.tile == 0)
    out, res = solver.run_batch(cfg, nx, ic)   # tpb = 0: uses the tuned tile
    assert res.tile == t.tile
    np.testing.assert_array_equal(out, _oracle_each(oracle, 1, 8, nx, ic, 0.005, 96))


def test_ensemble_rejects_bad_tile(sw, solver):
    nx = np.array([1024, 96], dtype=np.int64)
    cfg = sw.make_config(1, 8, alg=1, tpb=64, dt=0.005, time_mode=sw.TIME_STEPS, n_steps=8)
    with pytest.raises(sw.NativeError) as e:
        solver.run_batch(cfg, nx, np.zeros(int(nx.sum())))
    assert e.value.code == -2


def test_ensemble_applies_the_single_run_checks_to_every_domain(sw, solver):
    """sw_validate's checks hold for ensembles too: an Euler ensemble of uneven
    lengths must state dx (the default 1/(nx-2) differs per domain), Euler's
    stability limit applies, and the problem's boundary condition and flags
    are checked -- each rejected before any launch."""
    nx = np.array([256, 512], dtype=np.int64)
    ic = np.zeros(int(nx.sum()) * 3)
    cases = [
        (dict(problem=2, dt=1e-5), -1),                     # uneven Euler lengths, dx from nx: refused
        (dict(problem=2, dt=0.5 / 254, dx=1.0 / 254), -3),  # dt/dx = 0.5 > 0.21: unstable
        (dict(problem=1, bc=sw.BC_MIRROR, dt=0.005), -1),   # KS is periodic only
        (dict(problem=0, flags=sw.FLAG_KS_DIVIDE, dt=0.004), -1),  # the divide flag is KS's
    ]
    for over, code in cases:
        problem = over.pop("problem")
        cfg = sw.make_config(problem, 8, alg=1, tpb=64, time_mode=sw.TIME_STEPS, n_steps=8, **over)
        state = ic if problem == 2 else np.zeros(int(nx.sum()))
        with pytest.raises(sw.NativeError) as e:
            solver.run_batch(cfg, nx, state)
        assert e.value.code == code, (problem, over)
