"""The KS closure on the GPU: tensor-core forward and backward against the
float64 oracle (oracle/closure.py, same BF16 rounding points), the fused
coarse step, and what training on the solver's own fine trajectories gains
over the plain coarse step."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def cl():
    return importlib.import_module("1dsweptcuda_gb300.closure")


def _theta(seed, oracle_closure):
    th = oracle_closure.init(seed).astype(np.float64)
    rng = np.random.default_rng(seed + 100)
    th[5344:5504] = rng.standard_normal(160) * 0.1   # a non-trivial output layer
    th[160:192] = rng.standard_normal(32) * 0.1      # biases
    th[5312:5344] = rng.standard_normal(32) * 0.1
    th[5504] = 0.05
    th[5505] = 0.5      # output scale
    return th.astype(np.float32)


def test_infer_matches_oracle(sw, solver, cl):
    from oracle import closure as ocl
    th = _theta(1, ocl)
    rng = np.random.default_rng(2)
    u = (rng.standard_normal((3, 384)) * 1.5).astype(np.float32)
    c = cl.Closure(solver, th)
    got = c.infer(torch.from_numpy(u).cuda()).cpu().numpy().astype(np.float64)
    want = ocl.forward(th.astype(np.float64), u.astype(np.float64))
    err = np.abs(got - want).max() / np.abs(want).max()
    assert err < 5e-3, err


def test_grad_matches_oracle(sw, solver, cl):
    from oracle import closure as ocl
    th = _theta(3, ocl)
    rng = np.random.default_rng(4)
    u = (rng.standard_normal((4, 256)) * 1.5).astype(np.float32)
    tgt = (rng.standard_normal((4, 256)) * 0.05).astype(np.float32)
    c = cl.Closure(solver, th)
    g, loss = c.grad(torch.from_numpy(u).cuda(), torch.from_numpy(tgt).cuda())
    g = g.cpu().numpy().astype(np.float64)
    want_loss, want = ocl.loss_and_grad(th.astype(np.float64), u.astype(np.float64), tgt.astype(np.float64))
    assert abs(loss - want_loss) / want_loss < 1e-3
    rel = np.linalg.norm(g - want) / np.linalg.norm(want)
    assert rel < 3e-2, rel
    # every layer's gradient agrees on its own (not only the dominant one)
    assert g[5505] == 0.0   # the output scale is not trained
    for lo, hi in ((0, 160), (160, 192), (192, 5312), (5312, 5344), (5344, 5504), (5504, 5505)):
        r = np.linalg.norm(g[lo:hi] - want[lo:hi]) / (np.linalg.norm(want[lo:hi]) + 1e-30)
        assert r < 5e-2, (lo, hi, r)


def test_minibatch_rows_select_samples(sw, solver, cl):
    from oracle import closure as ocl
    th = _theta(5, ocl)
    rng = np.random.default_rng(6)
    u = torch.from_numpy((rng.standard_normal((6, 128))).astype(np.float32)).cuda()
    tgt = torch.from_numpy((rng.standard_normal((6, 128)) * 0.1).astype(np.float32)).cuda()
    c = cl.Closure(solver, th)
    g_rows, l_rows = c.grad(u, tgt, rows=[4, 1])
    g_sub, l_sub = c.grad(u[[4, 1]].contiguous(), tgt[[4, 1]].contiguous())
    assert torch.equal(g_rows, g_sub)
    assert abs(l_rows - l_sub) <= 1e-6 * l_sub   # the loss is summed with float atomics


def test_step_without_closure_is_classic_ks(sw, solver, cl):
    """The fused kernel with the closure off is the classic coarse KS step, bit for bit."""
    rng = np.random.default_rng(8)
    u = (rng.standard_normal((5, 1024))).astype(np.float32)
    c = cl.Closure(solver)
    t = torch.from_numpy(u.copy()).cuda()
    c.step(t, 7, use_closure=False)
    cfg = sw.make_config(sw.KS, 4, alg=sw.ALG_CLASSIC, tpb=128, dt=cl.COARSE_DT, dx=cl.COARSE_DX,
                         time_mode=sw.TIME_STEPS, n_steps=7)
    want, _ = solver.run_batch(cfg, np.full(5, 1024, dtype=np.int64), u.ravel())
    np.testing.assert_array_equal(t.cpu().numpy().ravel(), want)


def test_step_with_closure_adds_the_correction(sw, solver, cl):
    from oracle import closure as ocl
    th = _theta(9, ocl)
    rng = np.random.default_rng(10)
    u = torch.from_numpy((rng.standard_normal((3, 1024))).astype(np.float32)).cuda()
    c = cl.Closure(solver, th)
    a = u.clone()
    c.step(a, 1, use_closure=True)
    b = u.clone()
    c.step(b, 1, use_closure=False)
    assert torch.equal(a, b + c.infer(u))


def test_training_gains_over_plain_coarse_step(sw, solver, cl):
    """Trained on the fine solver's own trajectories, the closure removes most of
    the coarse step's defect on held-out trajectories and keeps the coarse run
    closer to the coarse-grained fine solution than the plain coarse step."""
    c = cl.Closure(solver, seed=0)
    spin = cl.CHAOS_SPINUP
    x, y = cl.make_training_data(solver, c, n_traj=96, snapshots=24, interval=10, seed=11, spinup=spin)
    c.calibrate(y)
    losses = c.train(x, y, steps=600, batch=32, lr=2e-3, seed=3)
    assert losses[-20:].mean() < 0.5 * losses[:5].mean()
    hx, hy = cl.make_training_data(solver, c, n_traj=16, snapshots=4, interval=10, seed=99, spinup=spin)
    resid = (hy - c.infer(hx)).pow(2).sum() / hy.pow(2).sum()
    assert float(resid) < 0.5, float(resid)
    # 25 coarse steps (t = 0.5) from held-out chaotic states against the coarse-grained fine run
    fine = cl.fine_ensemble(16, seed=123)
    cl.advance_fine(solver, fine, spin * cl.FACTOR)
    start = cl.coarse_grain(solver, fine)
    cl.advance_fine(solver, fine, 25 * cl.FACTOR)
    truth = cl.coarse_grain(solver, fine)
    plain, learned = start.clone(), start.clone()
    c.step(plain, 25, use_closure=False)
    c.step(learned, 25, use_closure=True)
    e_plain, e_learned = cl.rel_l2(plain, truth), cl.rel_l2(learned, truth)
    assert e_learned < 0.7 * e_plain, (e_learned, e_plain)


def test_adaptive_fallback_gives_the_fine_solution(sw, solver, cl):
    """run_adaptive with tau = 0: the first judged segment already fails, the
    run falls back, and the result is the coarse-grained fine solution from
    the exact start, bit for bit."""
    fine0 = cl.fine_ensemble(64, seed=321)
    c = cl.Closure(solver, seed=0)
    u, info = cl.run_adaptive(solver, c, fine0, coarse_steps=20, segment=10, tau=0.0, shadow_every=32)
    assert info["fallback"] and info["closure"] + info["plain"] == 0
    assert info["shadow_domains"] == 2
    f = fine0.clone()
    cl.advance_fine(solver, f, 20 * cl.FACTOR)
    assert torch.equal(u, cl.coarse_grain(solver, f))


def test_adaptive_judge_is_the_fine_solution_of_its_sample(sw, solver, cl):
    """On the smooth ensemble (from the IC) the judge picks the plain step
    over an untrained closure in every segment, nothing falls back, the
    certificate is the true error of the sampled domains, and every domain's
    error stays within the tolerance."""
    fine0 = cl.fine_ensemble(64, seed=77)
    c = cl.Closure(solver, seed=0)          # untrained: its correction is noise
    steps, tau = 100, 1e-3
    u, info = cl.run_adaptive(solver, c, fine0, coarse_steps=steps, segment=25, tau=tau, shadow_every=16)
    assert not info["fallback"] and info["plain"] == 4 and info["closure"] == 0
    assert all(r["used"] == "plain" and r["err"] < r["err_other"] for r in info["log"])
    truth = fine0.clone()
    cl.advance_fine(solver, truth, steps * cl.FACTOR)
    ref = cl.coarse_grain(solver, truth)
    err = (u.double() - ref.double()).norm(dim=1) / ref.double().norm(dim=1)
    sample = cl.shadow_domains(64, 16, 0)
    assert abs(float(err[sample].max()) - info["shadow_max_rel_l2"]) < 1e-12
    assert abs(float(err[sample].mean()) - info["shadow_mean_rel_l2"]) < 1e-12
    assert float(err.max()) < tau, err


def test_largest_certified_horizon(cl):
    rows = [{"tf": 10, "rel_l2_plain": 1e-5, "speedup_plain_vs_fine": 12, "rel_l2_closure": 1e-2,
             "speedup_closure_vs_fine": 6, "rel_l2_adaptive": 1e-5, "speedup_adaptive_vs_fine": 9, "fallback": False},
            {"tf": 30, "rel_l2_plain": 5e-4, "speedup_plain_vs_fine": 12, "rel_l2_closure": 1e-1,
             "speedup_closure_vs_fine": 6, "rel_l2_adaptive": 5e-4, "speedup_adaptive_vs_fine": 9, "fallback": False},
            {"tf": 40, "rel_l2_plain": 2e-3, "speedup_plain_vs_fine": 12, "rel_l2_closure": 1.0,
             "speedup_closure_vs_fine": 6, "rel_l2_adaptive": 0.0, "speedup_adaptive_vs_fine": 0.9, "fallback": True}]
    assert cl.largest_certified(rows, 1e-3) == {"plain": 30, "closure": None, "adaptive": 30}


def test_step_without_closure_needs_no_parameters(sw, solver, cl):
    """sw_closure_step with the closure off takes a null theta (nothing reads it)."""
    import ctypes as C
    rng = np.random.default_rng(12)
    u = (rng.standard_normal((2, 1024))).astype(np.float32)
    t = torch.from_numpy(u.copy()).cuda()
    c = cl.Closure(solver)
    cfg = c.coarse_config()
    res = sw.Result()
    rc = sw.library().sw_closure_step(solver._ctx, C.byref(cfg), None, C.c_void_p(t.data_ptr()), 2, 1024, 3, 0,
                                      C.byref(res))
    assert rc == 0
    want = torch.from_numpy(u.copy()).cuda()
    c.step(want, 3, use_closure=False)
    assert torch.equal(t, want)
