"""SW_FLAG_KS_DIVIDE on the GPU (the reference's DIVISE build,
KS1D_SweptShared.cu:111-132): classic, swept, the 32-cell variant and an
ensemble, each equal bit for bit to the oracle's divide form.  At dx = 0.3 the
divisors are not powers of two, so the divide build's roundings differ from the
reciprocal build's and the comparison tells the two apart; the same cases
without the flag cover the library's unfused reciprocal path."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KS = 1
ens = importlib.import_module("1dsweptcuda_gb300.ensemble")


def _ic(prec, nx, seed):
    rng = np.random.default_rng(seed)
    x = np.arange(nx)
    u = np.cos(2 * np.pi * 5 * x / nx) + 0.1 * rng.standard_normal(nx)
    return u.astype(np.float64 if prec == 8 else np.float32)


@pytest.mark.parametrize("prec", [8, 4])
@pytest.mark.parametrize("dx, dt", [(0.5, 0.005), (0.3, 5e-4)])
@pytest.mark.parametrize("divide", [True, False])
def test_single_domain(sw, solver, oracle, prec, dx, dt, divide):
    nx, tpb = 2048, 128
    ic = _ic(prec, nx, 4)
    c = oracle.ks_consts(prec, nx, dt, dx=dx, divide=divide)
    flags = sw.FLAG_KS_DIVIDE if divide else 0
    for steps in (32, 77):
        want = oracle.classic(c, ic, steps)
        for alg in (sw.ALG_CLASSIC, sw.ALG_SWEPT, sw.ALG_VARIANT):
            cfg = sw.make_config(KS, prec, alg=alg, nx=nx, tpb=tpb, dt=dt, dx=dx, flags=flags,
                                 time_mode=sw.TIME_STEPS, n_steps=steps)
            got, res, _ = solver.run(cfg, ic)
            assert res.n_steps == steps
            np.testing.assert_array_equal(got, want, err_msg="alg %d steps %d" % (alg, steps))


@pytest.mark.parametrize("prec", [8, 4])
def test_divide_differs_from_reciprocal_at_dx_03(sw, solver, prec):
    nx, dt, dx = 1024, 5e-4, 0.3
    ic = _ic(prec, nx, 6)
    out = []
    for flags in (0, sw.FLAG_KS_DIVIDE):
        cfg = sw.make_config(KS, prec, alg=sw.ALG_SWEPT, nx=nx, tpb=64, dt=dt, dx=dx, flags=flags,
                             time_mode=sw.TIME_STEPS, n_steps=64)
        out.append(solver.run(cfg, ic)[0])
    assert not np.array_equal(out[0], out[1])


@pytest.mark.parametrize("alg", [0, 1, 2])
def test_ensemble(sw, solver, oracle, alg):
    nx, ic = ens.make_ensemble(n_domains=12, lo=7, hi=11, seed=8)
    dx, dt, steps = 0.3, 5e-4, 44
    cfg = sw.make_config(KS, 8, alg=alg, tpb=64, dt=dt, dx=dx, flags=sw.FLAG_KS_DIVIDE,
                         time_mode=sw.TIME_STEPS, n_steps=steps)
    out, res = solver.run_batch(cfg, nx, ic)
    assert res.n_steps == steps
    want = ens.concat([oracle.classic(oracle.ks_consts(8, int(n), dt, dx=dx, divide=True), part, steps)
                       for part, n in zip(ens.split(ic, nx, 1), nx)])
    np.testing.assert_array_equal(out, want)
