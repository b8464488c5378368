"""Config 4 at full size: the seeded 4096-domain KS ensemble, nx = 2^e with e
uniform on 10..16 (7.6e7 cells), dx = 0.5, dt = 0.005.  FP32: swept (the
autotuned tile), the persistent variant and classic are equal bit for bit
over two full cycles of the largest tile plus a remainder.  FP64: swept over
two cycles plus a remainder, eight sampled domains equal the oracle run on
each domain alone, bit for bit."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ens = importlib.import_module("1dsweptcuda_gb300.ensemble")


def test_fp32_full_ensemble_swept_variant_classic_identical(sw, solver):
    torch = pytest.importorskip("torch")
    nx, u = ens.make_ensemble(n_domains=4096)
    steps = 2 * 128 + 37       # two cycles of a 1024-cell tile (128 steps each), then 37 classic steps
    finals = {}
    for alg, tpb in ((sw.ALG_SWEPT, 1024), (sw.ALG_VARIANT, 1024), (sw.ALG_CLASSIC, 256)):
        cfg = sw.make_config(sw.KS, 4, alg=alg, tpb=tpb, dt=0.005, time_mode=sw.TIME_STEPS, n_steps=steps)
        st = torch.from_numpy(u.astype(np.float32)).cuda()
        res = solver.run_batch_device(cfg, nx, st.data_ptr())
        assert res.n_steps == steps
        finals[alg] = st
    assert torch.isfinite(finals[sw.ALG_SWEPT]).all()
    assert torch.equal(finals[sw.ALG_SWEPT], finals[sw.ALG_CLASSIC])
    assert torch.equal(finals[sw.ALG_VARIANT], finals[sw.ALG_CLASSIC])


def test_fp64_full_ensemble_sampled_domains_equal_the_oracle(sw, solver, oracle):
    torch = pytest.importorskip("torch")
    nx, u = ens.make_ensemble(n_domains=4096)
    steps = 2 * 64 + 13        # two cycles of a 512-cell tile (64 steps each), then 13 classic steps
    cfg = sw.make_config(sw.KS, 8, alg=sw.ALG_SWEPT, tpb=512, dt=0.005, time_mode=sw.TIME_STEPS, n_steps=steps)
    st = torch.from_numpy(u.copy()).cuda()
    solver.run_batch_device(cfg, nx, st.data_ptr())
    got = ens.split(st.cpu().numpy(), nx)
    parts = ens.split(u, nx)
    rng = np.random.default_rng(4096)
    pick = list(rng.choice(4096, size=6, replace=False)) + [int(np.argmax(nx)), int(np.argmin(nx))]
    for d in pick:
        c = oracle.reference_consts(oracle.KS, 8, int(nx[d]), 0.005)
        np.testing.assert_array_equal(got[d], oracle.classic(c, parts[d], steps), err_msg="domain %d" % d)
