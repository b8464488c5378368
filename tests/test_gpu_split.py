"""The split domain on the GPU: P parts of one periodic domain, each advanced by
sw_swept_pass as a periodic domain of its own on the device, with the ring
exchange done by device copies (split.run_local), equal bit for bit to the
single-domain run (sw_run_device).  Also sw_swept_pass alone: up, diamonds and
down launched one by one equal the library's own swept run."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
split = importlib.import_module("1dsweptcuda_gb300.split")


def _ic(sw, cfg):
    if cfg.problem == sw.HEAT:
        x = np.arange(cfg.nx)
        return (50.0 + 100.0 * np.sin(2 * np.pi * x / cfg.nx)).astype(np.float64 if cfg.precision == 8 else np.float32)
    return sw.initial_condition(cfg)


@pytest.mark.parametrize("problem,prec,nx,tpb,parts,steps", [
    (1, 8, 1 << 16, 256, 2, 32 * 9),    # KS FP64: odd diamond count, the down-triangle moves cells
    (1, 8, 1 << 16, 256, 4, 32 * 8),
    (1, 4, 1 << 18, 1024, 4, 128 * 5),  # FP32 4-cells-per-thread tiles
    (1, 8, 1 << 20, 256, 8, 32 * 7),    # eight parts of the benchmark's domain
    (0, 8, 1 << 14, 128, 2, 64 * 7),    # Heat, periodic ends
])
def test_split_parts_equal_the_single_domain_run(sw, solver, problem, prec, nx, tpb, parts, steps):
    bc = sw.BC_PERIODIC if problem == sw.HEAT else sw.BC_DEFAULT
    dt = 0.004 if problem == sw.HEAT else 0.005
    cfg = sw.make_config(problem, prec, alg=sw.ALG_SWEPT, nx=nx, tpb=tpb, dt=dt, bc=bc, time_mode=sw.TIME_STEPS,
                         n_steps=steps)
    ic = _ic(sw, cfg)
    whole = torch.from_numpy(ic.copy()).cuda()
    solver.run_device(cfg, whole.data_ptr())
    n = nx // parts
    states = [torch.from_numpy(ic[r * n:(r + 1) * n].copy()).cuda() for r in range(parts)]
    passes = split.run_local(solver, cfg, states, steps)
    torch.cuda.synchronize()
    assert passes == steps // split.steps_per_diamond(problem, tpb) + 1
    np.testing.assert_array_equal(torch.cat(states).cpu().numpy(), whole.cpu().numpy())


def test_single_passes_equal_the_swept_run(sw, solver):
    nx, tpb, steps = 1 << 15, 128, 16 * 6
    cfg = sw.make_config(sw.KS, 8, alg=sw.ALG_SWEPT, nx=nx, tpb=tpb, dt=0.005, time_mode=sw.TIME_STEPS,
                         n_steps=steps)
    ic = sw.initial_condition(cfg)
    want = torch.from_numpy(ic.copy()).cuda()
    solver.run_device(cfg, want.data_ptr())
    st = torch.from_numpy(ic.copy()).cuda()
    slots = torch.empty(2 * nx, dtype=torch.float64, device="cuda")
    for mode, phase in split.schedule(steps, split.steps_per_diamond(sw.KS, tpb)):
        solver.swept_pass(cfg, mode, phase, st.data_ptr(), slots.data_ptr())
    torch.cuda.synchronize()
    np.testing.assert_array_equal(st.cpu().numpy(), want.cpu().numpy())


def test_swept_pass_rejects_bad_requests(sw, solver):
    cfg = sw.make_config(sw.KS, 8, alg=sw.ALG_SWEPT, nx=1024, tpb=128, dt=0.005)
    st = torch.zeros(1024, dtype=torch.float64, device="cuda")
    sl = torch.zeros(2048, dtype=torch.float64, device="cuda")
    for mode, phase in ((0, 1), (3, 0), (1, 2)):
        with pytest.raises(sw.NativeError) as e:
            solver.swept_pass(cfg, mode, phase, st.data_ptr(), sl.data_ptr())
        assert e.value.code == -1
    classic = sw.make_config(sw.KS, 8, alg=sw.ALG_CLASSIC, nx=1024, tpb=128, dt=0.005)
    with pytest.raises(sw.NativeError) as e:
        solver.swept_pass(classic, 1, 1, st.data_ptr(), sl.data_ptr())
    assert e.value.code == -8
