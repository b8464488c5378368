"""sw_run_device_noalloc: the swept run for callers that cannot allocate
device memory (their GPU memory is sized once up front and owned by their own
arena, or they step the solver where cudaMalloc is not allowed).  Its scratch
is a fixed array inside the library instead of context buffers.

Called here through the C ABI (ctypes) on a device state and compared with
the existing entry point sw_run_device on the same input: bit-identical, the
tolerance every parity test in this suite uses, on two calls in a row (the
second call reuses the array the first one left behind).  This file is
collected last so that a stop-at-first-failure run has already run every
other test; it also passes alone in a fresh process."""
import ctypes as C
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _device_ic(sw, cfg):
    ic = sw.initial_condition(cfg)
    if cfg.problem == sw.EULER:
        dev = np.zeros((cfg.nx, 4), dtype=ic.dtype)
        dev[:, :3] = ic.reshape(-1, 3)
        ic = dev.ravel()
    return ic


@pytest.mark.parametrize("problem,prec,nx,tpb,dt,steps,threads", [
    (1, 8, 1 << 20, 256, 0.005, 200, 0),      # the benchmark's KS domain, the largest FP64 size the scratch holds
    (1, 4, 1 << 16, 128, 0.005, 101, 0),      # remainder steps use the scratch work row
    (0, 8, 4096, 128, 0.004, 333, 0),         # Heat: odd remainder ends in the work row
    (2, 8, 1 << 14, 256, 0.1 / 16382, 97, 0),  # Euler, 4 values per cell
    (1, 4, 1 << 20, 1024, 0.005, 515, 0),     # FP32 KS, 1024 tiles of 1024 cells, 4 cells per thread
    (1, 4, 1 << 18, 256, 0.005, 203, 0),      # FP32 KS, 1024 tiles: four tiles per block (grouped slots)
    (1, 8, 1 << 16, 256, 0.005, 131, 128),    # a non-default threads per block: two cells per thread
])
def test_noalloc_matches_sw_run_device_twice(sw, solver, problem, prec, nx, tpb, dt, steps, threads):
    torch = pytest.importorskip("torch")
    lib = sw.library()
    cfg = sw.make_config(problem, prec, alg=sw.ALG_SWEPT, nx=nx, tpb=tpb, dt=dt, time_mode=sw.TIME_STEPS,
                         n_steps=steps)
    cfg.threads = threads
    ic = _device_ic(sw, cfg)
    want = torch.from_numpy(ic.copy()).cuda()
    solver.run_device(cfg, want.data_ptr())
    want = want.cpu().numpy()
    stream = torch.cuda.current_stream()
    for call in range(2):
        st = torch.from_numpy(ic.copy()).cuda()
        torch.cuda.synchronize()
        rc = lib.sw_run_device_noalloc(C.byref(cfg), C.c_void_p(st.data_ptr()),
                                       C.c_void_p(stream.cuda_stream) if stream.cuda_stream else None)
        assert rc == 0, (call, rc)
        torch.cuda.synchronize()
        got = st.cpu().numpy()
        np.testing.assert_array_equal(got, want, err_msg="call %d" % call)


def test_noalloc_rejects_sizes_beyond_the_scratch(sw):
    native = importlib.import_module("1dsweptcuda_gb300.native")
    lib = sw.library()
    # FP64 KS needs 3 x 8 bytes per cell: 2^20 cells fit in 24 MiB, 2^21 do not
    big = sw.make_config(1, 8, alg=sw.ALG_SWEPT, nx=1 << 21, tpb=256, dt=0.005, time_mode=sw.TIME_STEPS, n_steps=32)
    assert 3 * 8 * (1 << 21) > native.NOALLOC_SCRATCH_BYTES
    assert lib.sw_run_device_noalloc(C.byref(big), C.c_void_p(1), None) == -2   # SW_ERR_SIZE, before any launch
    classic = sw.make_config(1, 8, alg=sw.ALG_CLASSIC, nx=1024, tpb=256, dt=0.005, time_mode=sw.TIME_STEPS,
                             n_steps=32)
    assert lib.sw_run_device_noalloc(C.byref(classic), C.c_void_p(1), None) == -8  # swept only


def test_noalloc_rejects_a_state_that_is_not_device_memory(sw):
    """A host buffer (or any pointer that is not device memory of the current
    device) is turned away before a kernel could touch it."""
    lib = sw.library()
    cfg = sw.make_config(1, 8, alg=sw.ALG_SWEPT, nx=1024, tpb=256, dt=0.005, time_mode=sw.TIME_STEPS, n_steps=32)
    host = np.zeros(1024, dtype=np.float64)
    assert lib.sw_run_device_noalloc(C.byref(cfg), host.ctypes.data_as(C.c_void_p), None) == -1  # SW_ERR_ARG
