"""The KS DIVISE build (KS1D_SweptShared.cu:111-132, 904-914) on the CPU: the
constants the library derives for SW_FLAG_KS_DIVIDE, its argument checks, and
the oracle's divide form.  At the reference's dx = 0.5 every divisor is a power
of two, so dividing and multiplying by the reciprocal give the same bits; the
GPU paths are checked against the oracle in test_gpu_ks_divide.py."""
import numpy as np
import pytest

KS, HEAT, EULER = 1, 0, 2


@pytest.mark.parametrize("prec", [8, 4])
@pytest.mark.parametrize("dx", [0.5, 0.3, 2.0])
@pytest.mark.parametrize("divide", [False, True])
def test_constants_match_oracle(sw, oracle, prec, dx, divide):
    cfg = sw.make_config(KS, prec, nx=1024, tpb=64, dt=1e-3, dx=dx, flags=sw.FLAG_KS_DIVIDE if divide else 0)
    k = sw.constants(cfg)
    o = oracle.ks_consts(prec, 1024, 1e-3, dx=dx, divide=divide)
    for f in ("dx_times4", "dx2", "dx4", "dt", "dt_half"):
        assert getattr(k, f) == getattr(o, f), f


def test_flag_checks(sw):
    assert sw.validate(sw.make_config(KS, 8, flags=sw.FLAG_KS_DIVIDE)) == 0
    for problem in (HEAT, EULER):
        assert sw.validate(sw.make_config(problem, 8, flags=sw.FLAG_KS_DIVIDE)) == -1  # SW_ERR_ARG
    assert sw.validate(sw.make_config(KS, 8, flags=4)) == -1   # no such flag


@pytest.mark.parametrize("prec", [8, 4])
def test_oracle_divide_form(oracle, prec):
    nx, steps = 512, 60
    ic = oracle.reference_ic(KS, prec, nx)
    # dx = 0.5: the same bits as the reciprocal build, which the golden vectors pin
    mul = oracle.classic(oracle.reference_consts(KS, prec, nx, 0.005), ic, steps)
    div = oracle.classic(oracle.ks_consts(prec, nx, 0.005, divide=True), ic, steps)
    np.testing.assert_array_equal(div, mul)
    # dx = 0.3: the two builds round differently, by a few units in the last place
    mul = oracle.classic(oracle.ks_consts(prec, nx, 5e-4, dx=0.3), ic, steps)
    div = oracle.classic(oracle.ks_consts(prec, nx, 5e-4, dx=0.3, divide=True), ic, steps)
    assert not np.array_equal(div, mul)
    eps = np.finfo(div.dtype).eps
    assert float(np.abs(div.astype(np.float64) - mul).max()) < 1e3 * eps * float(np.abs(mul).max())
