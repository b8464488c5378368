"""ctypes binding of libswept1d (include/swept1d.h).

Mirrors the reference's run interface: a run is configured by the same values
its programs take on the command line (nx, tpb, dt, tf, freq, alg) and returns
the final state plus the snapshots the reference writes to its .dat file.
There is no fallback: every call goes to the CUDA library, and a missing
library is an error.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path
from typing import Callable

import numpy as np

HEAT, KS, EULER = 0, 1, 2
ALG_CLASSIC, ALG_SWEPT, ALG_VARIANT, ALG_SELFTEST = 0, 1, 2, 3
BC_DEFAULT, BC_MIRROR, BC_PERIODIC, BC_DIRICHLET = 0, 1, 2, 3
TIME_REFERENCE, TIME_STEPS = 0, 1
FLAG_KS_DIVIDE = 1  # sw_config.flags: KS divides by 4dx, dx^2, dx^4 (the reference's DIVISE build)
FLAG_HOST_TILE = 2  # sw_config.flags: the hybrid variant, each phase-1 pass's wrapping tile on the host
COMPONENTS = {HEAT: 1, KS: 1, EULER: 3}
PROBLEM_NAMES = {HEAT: "Heat", KS: "KS", EULER: "Euler"}

ERRORS = {0: "SW_OK", -1: "SW_ERR_ARG", -2: "SW_ERR_SIZE", -3: "SW_ERR_UNSTABLE", -4: "SW_ERR_CUDA",
          -5: "SW_ERR_NOMEM", -6: "SW_ERR_IO", -7: "SW_ERR_TIMEOUT", -8: "SW_ERR_UNSUPPORTED",
          -9: "SW_ERR_CALLBACK", -10: "SW_ERR_USAGE"}

EXPORTED = ["sw_abi_version", "sw_strerror", "sw_ctx_create", "sw_ctx_destroy", "sw_ctx_last_error",
            "sw_config_init", "sw_validate", "sw_constants_of", "sw_initial_condition", "sw_run",
            "sw_run_device", "sw_plan", "sw_cli_main", "sw_run_batch", "sw_run_batch_device",
            "sw_query_tuning", "sw_run_device_noalloc", "sw_closure_infer", "sw_closure_step",
            "sw_closure_grad", "sw_closure_adam", "sw_closure_train", "sw_coarse_grain", "sw_wait_probe",
            "sw_fp64_rates", "sw_swept_pass", "sw_closure_adaptive"]
CLOSURE_PARAMS = 5506
CUDA_STREAM_LEGACY = 1  # cudaStreamLegacy: the legacy default stream (a stream argument of 0 means the context's own)


def torch_stream() -> int:
    """The handle of torch's current CUDA stream as the C ABI takes it: torch's
    default stream is the legacy default stream, handle 0, which the ABI reads
    as "the context's stream"; cudaStreamLegacy names it instead."""
    import torch
    return torch.cuda.current_stream().cuda_stream or CUDA_STREAM_LEGACY
NOALLOC_SCRATCH_BYTES = 24 * 1024 * 1024


class Config(C.Structure):
    _fields_ = [
        ("problem", C.c_int32), ("precision", C.c_int32), ("alg", C.c_int32), ("bc", C.c_int32),
        ("nx", C.c_int64), ("tpb", C.c_int32), ("time_mode", C.c_int32),
        ("dt", C.c_double), ("tf", C.c_double), ("freq", C.c_double), ("n_steps", C.c_int64),
        ("dx", C.c_double), ("alpha", C.c_double), ("gamma", C.c_double),
        ("left", C.c_double * 3), ("right", C.c_double * 3),
        ("threads", C.c_int32), ("flags", C.c_int32),
    ]


class Constants(C.Structure):
    _fields_ = [
        ("fourier", C.c_double), ("fourier_two", C.c_double),
        ("dx_times4", C.c_double), ("dx2", C.c_double), ("dx4", C.c_double), ("dt", C.c_double),
        ("dt_half", C.c_double), ("gam", C.c_double), ("mgam", C.c_double), ("dt_dx", C.c_double),
        ("bd", C.c_double * 6), ("lx", C.c_double), ("dx", C.c_double),
    ]


class Result(C.Structure):
    _fields_ = [
        ("t_final", C.c_double), ("n_steps", C.c_int64), ("elapsed_ms", C.c_double),
        ("us_per_step", C.c_double), ("kernel_ms", C.c_double), ("launches", C.c_int64),
        ("snapshots", C.c_int32), ("tile", C.c_int32),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class AdaptiveInfo(C.Structure):
    _fields_ = [("closure_segments", C.c_int32), ("plain_segments", C.c_int32), ("fallback", C.c_int32),
                ("n_shadow", C.c_int32), ("n_log", C.c_int32), ("shadow_mean_rel_l2", C.c_double),
                ("shadow_max_rel_l2", C.c_double)]


class PlanInfo(C.Structure):
    _fields_ = [("t_final", C.c_double), ("n_steps", C.c_int64), ("n_snapshots", C.c_int32),
                ("tile", C.c_int32), ("launches", C.c_int64)]


class Tuning(C.Structure):
    _fields_ = [("tile", C.c_int32), ("threads", C.c_int32), ("cell_updates_per_s", C.c_double),
                ("n_candidates", C.c_int32), ("cand_tile", C.c_int32 * 48), ("cand_threads", C.c_int32 * 48),
                ("cand_rate", C.c_double * 48)]

    def candidates(self) -> list[tuple[int, int, float]]:
        return [(self.cand_tile[i], self.cand_threads[i], self.cand_rate[i]) for i in range(self.n_candidates)]


SNAPSHOT_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_double, C.c_void_p, C.c_int64)


class NativeError(RuntimeError):
    def __init__(self, code: int, message: str = ""):
        self.code = code
        super().__init__("%s (%d)%s" % (ERRORS.get(code, "unknown"), code, (": " + message) if message else ""))


def library_path() -> Path:
    return Path(__file__).resolve().parent / "lib" / "libswept1d.so"


_lib = None


def library():
    """Load libswept1d.so (built by build.py / __graft_entry__.build()); raise if absent."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not path.exists():
        raise ImportError("libswept1d.so not built (%s); run python 1dsweptcuda_gb300/build.py" % path)
    L = C.CDLL(str(path))
    cp, rp, kp = C.POINTER(Config), C.POINTER(Result), C.POINTER(Constants)
    L.sw_abi_version.restype = C.c_int
    L.sw_strerror.argtypes = [C.c_int]
    L.sw_strerror.restype = C.c_char_p
    L.sw_ctx_create.argtypes = [C.c_int, C.POINTER(C.c_void_p)]
    L.sw_ctx_destroy.argtypes = [C.c_void_p]
    L.sw_ctx_last_error.argtypes = [C.c_void_p]
    L.sw_ctx_last_error.restype = C.c_char_p
    L.sw_config_init.argtypes = [cp, C.c_int, C.c_int]
    L.sw_validate.argtypes = [cp]
    L.sw_constants_of.argtypes = [cp, kp]
    L.sw_initial_condition.argtypes = [cp, C.c_void_p]
    L.sw_run.argtypes = [C.c_void_p, cp, C.c_void_p, C.c_void_p, SNAPSHOT_FN, C.c_void_p, rp]
    L.sw_run_device.argtypes = [C.c_void_p, cp, C.c_void_p, C.c_void_p, rp]
    L.sw_cli_main.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_char_p)]
    L.sw_plan.argtypes = [cp, C.POINTER(PlanInfo), C.POINTER(C.c_double), C.POINTER(C.c_int64), C.c_int32]
    i64p = C.POINTER(C.c_int64)
    L.sw_run_batch.argtypes = [C.c_void_p, cp, C.c_int32, i64p, C.c_void_p, C.c_void_p, rp]
    L.sw_run_batch_device.argtypes = [C.c_void_p, cp, C.c_int32, i64p, C.c_void_p, C.c_void_p, rp]
    L.sw_query_tuning.argtypes = [C.c_void_p, cp, C.c_int32, i64p, C.POINTER(Tuning)]
    L.sw_run_device_noalloc.argtypes = [cp, C.c_void_p, C.c_void_p]
    vp = C.c_void_p
    L.sw_closure_infer.argtypes = [vp, vp, vp, vp, C.c_int32, C.c_int64]
    L.sw_closure_step.argtypes = [vp, cp, vp, vp, C.c_int32, C.c_int64, C.c_int64, C.c_int32, rp]
    L.sw_closure_grad.argtypes = [vp, vp, vp, vp, vp, C.c_int32, C.c_int64, vp]
    L.sw_closure_adam.argtypes = [vp, vp, vp, vp, vp, C.c_int32, C.c_float]
    L.sw_closure_train.argtypes = [vp, vp, vp, vp, C.c_int64, C.c_int64, C.c_int32, C.c_int32, C.c_float,
                                   C.c_uint64, C.POINTER(C.c_float)]
    L.sw_coarse_grain.argtypes = [vp, vp, vp, C.c_int64, C.c_int32]
    L.sw_wait_probe.argtypes = [vp, C.c_int64, C.POINTER(C.c_double)]
    dp = C.POINTER(C.c_double)
    L.sw_fp64_rates.argtypes = [vp, dp, dp, dp]
    L.sw_swept_pass.argtypes = [vp, cp, C.c_int32, C.c_int32, vp, vp, vp]
    L.sw_closure_adaptive.argtypes = [vp, vp, cp, cp, vp, vp, C.c_int32, C.c_int64, C.c_int32, C.c_int64, C.c_int64,
                                      C.c_double, C.c_int32, C.c_int32, vp, C.POINTER(AdaptiveInfo),
                                      C.POINTER(C.c_double), C.c_int32]
    for name in ("sw_ctx_create", "sw_ctx_destroy", "sw_config_init", "sw_validate", "sw_constants_of",
                 "sw_initial_condition", "sw_run", "sw_run_device", "sw_cli_main", "sw_plan", "sw_run_batch",
                 "sw_run_batch_device", "sw_query_tuning", "sw_run_device_noalloc", "sw_closure_infer",
                 "sw_closure_step", "sw_closure_grad", "sw_closure_adam", "sw_closure_train", "sw_coarse_grain",
                 "sw_fp64_rates", "sw_swept_pass", "sw_closure_adaptive"):
        getattr(L, name).restype = C.c_int
    _lib = L
    return L


def make_config(problem: int, precision: int = 8, **kw) -> Config:
    """A Config with the reference's defaults, then the given fields."""
    c = Config()
    rc = library().sw_config_init(C.byref(c), problem, precision)
    if rc:
        raise NativeError(rc)
    for k, v in kw.items():
        if k in ("left", "right"):
            for i in range(3):
                getattr(c, k)[i] = v[i]
        elif not hasattr(c, k):
            raise AttributeError("Config has no field %r" % k)
        else:
            setattr(c, k, v)
    return c


def validate(cfg: Config) -> int:
    return library().sw_validate(C.byref(cfg))


def constants(cfg: Config) -> Constants:
    k = Constants()
    rc = library().sw_constants_of(C.byref(cfg), C.byref(k))
    if rc:
        raise NativeError(rc)
    return k


def _dtype(cfg: Config):
    return np.float64 if cfg.precision == 8 else np.float32


def initial_condition(cfg: Config) -> np.ndarray:
    out = np.zeros(cfg.nx * COMPONENTS[cfg.problem], dtype=_dtype(cfg))
    rc = library().sw_initial_condition(C.byref(cfg), out.ctypes.data)
    if rc:
        raise NativeError(rc)
    return out


class Solver:
    """One device context (stream + reusable work buffers)."""

    def __init__(self, device: int = 0):
        self.device = device
        self._lib = library()
        self._ctx = C.c_void_p()
        rc = self._lib.sw_ctx_create(device, C.byref(self._ctx))
        if rc:
            raise NativeError(rc, "sw_ctx_create")

    def close(self) -> None:
        if self._ctx:
            self._lib.sw_ctx_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _err(self, rc: int, what: str) -> NativeError:
        msg = self._lib.sw_ctx_last_error(self._ctx)
        return NativeError(rc, "%s: %s" % (what, msg.decode() if msg else ""))

    def run(self, cfg: Config, ic: np.ndarray | None = None,
            on_snapshot: Callable[[float, np.ndarray], None] | None = None):
        """Host-to-host run (sw_run).  Returns (final_state, Result, snapshots),
        snapshots = [(t, state)] at the reference's output times."""
        dtype = _dtype(cfg)
        n = cfg.nx * COMPONENTS[cfg.problem]
        if ic is None:
            ic = initial_condition(cfg)
        ic = np.ascontiguousarray(ic, dtype=dtype)
        if ic.size != n:
            raise ValueError("initial condition has %d values, expected %d" % (ic.size, n))
        final = np.empty(n, dtype=dtype)
        snaps: list[tuple[float, np.ndarray]] = []

        def cb(_user, t, ptr, nx):
            arr = np.ctypeslib.as_array(C.cast(ptr, C.POINTER(C.c_double if dtype == np.float64 else C.c_float)),
                                        shape=(n,)).copy()
            snaps.append((t, arr))
            if on_snapshot is not None:
                on_snapshot(t, arr)
            return 0

        cbf = SNAPSHOT_FN(cb)
        res = Result()
        rc = self._lib.sw_run(self._ctx, C.byref(cfg), ic.ctypes.data, final.ctypes.data, cbf, None, C.byref(res))
        if rc:
            raise self._err(rc, "sw_run")
        return final, res, snaps

    def swept_pass(self, cfg: Config, mode: int, phase: int, state_ptr: int, slots_ptr: int, stream: int = 0) -> None:
        """sw_swept_pass: one up (0) / diamond (1) / down (2) launch over the
        domain's tiles on device state and slots (2 * nx cells); enqueued, not waited for."""
        rc = self._lib.sw_swept_pass(self._ctx, C.byref(cfg), int(mode), int(phase), C.c_void_p(state_ptr),
                                     C.c_void_p(slots_ptr), C.c_void_p(stream) if stream else None)
        if rc:
            raise self._err(rc, "sw_swept_pass")

    def run_device(self, cfg: Config, state_ptr: int, stream: int = 0) -> Result:
        """Device-resident run (sw_run_device) on a device pointer in device layout
        (Euler: 4 values per cell).  Blocks until the run completes."""
        res = Result()
        rc = self._lib.sw_run_device(self._ctx, C.byref(cfg), C.c_void_p(state_ptr),
                                     C.c_void_p(stream) if stream else None, C.byref(res))
        if rc:
            raise self._err(rc, "sw_run_device")
        return res


def _nx_array(nx):
    arr = np.ascontiguousarray(nx, dtype=np.int64)
    return arr, arr.ctypes.data_as(C.POINTER(C.c_int64))


class _BatchMixin:
    def run_batch(self, cfg: Config, nx, ic: np.ndarray) -> tuple[np.ndarray, Result]:
        """sw_run_batch: the domains' states concatenated (host layout) in, out."""
        arr, ptr = _nx_array(nx)
        n = int(arr.sum()) * COMPONENTS[cfg.problem]
        ic = np.ascontiguousarray(ic, dtype=_dtype(cfg))
        if ic.size != n:
            raise ValueError("ensemble state has %d values, expected %d" % (ic.size, n))
        out = np.empty_like(ic)
        res = Result()
        rc = self._lib.sw_run_batch(self._ctx, C.byref(cfg), len(arr), ptr, ic.ctypes.data, out.ctypes.data,
                                    C.byref(res))
        if rc:
            raise self._err(rc, "sw_run_batch")
        return out, res

    def run_batch_device(self, cfg: Config, nx, state_ptr: int, stream: int = 0) -> Result:
        arr, ptr = _nx_array(nx)
        res = Result()
        rc = self._lib.sw_run_batch_device(self._ctx, C.byref(cfg), len(arr), ptr, C.c_void_p(state_ptr),
                                           C.c_void_p(stream) if stream else None, C.byref(res))
        if rc:
            raise self._err(rc, "sw_run_batch_device")
        return res

    def tune(self, cfg: Config, nx) -> "Tuning":
        arr, ptr = _nx_array(nx)
        t = Tuning()
        rc = self._lib.sw_query_tuning(self._ctx, C.byref(cfg), len(arr), ptr, C.byref(t))
        if rc:
            raise self._err(rc, "sw_query_tuning")
        return t

    def wait_probe(self, limit_ns: int) -> tuple[int, float]:
        """sw_wait_probe: run the bounded wait on a flag nothing sets; returns
        (status code, milliseconds waited).  SW_ERR_TIMEOUT (-7) is the expected code."""
        ms = C.c_double(0.0)
        rc = self._lib.sw_wait_probe(self._ctx, int(limit_ns), C.byref(ms))
        return rc, ms.value


    def fp64_rates(self) -> dict:
        """sw_fp64_rates: measured FP64 fma / add / multiply issue rates (operations/s)."""
        f, a, m = C.c_double(), C.c_double(), C.c_double()
        rc = self._lib.sw_fp64_rates(self._ctx, C.byref(f), C.byref(a), C.byref(m))
        if rc:
            raise self._err(rc, "sw_fp64_rates")
        return {"fma": f.value, "add": a.value, "mul": m.value}


for _name in ("run_batch", "run_batch_device", "tune", "wait_probe", "fp64_rates"):
    setattr(Solver, _name, getattr(_BatchMixin, _name))


def run_device_noalloc(cfg: Config, state_ptr: int, stream: int = 0) -> None:
    """sw_run_device_noalloc: swept run on a device state using the library's
    fixed scratch array (no device allocation); enqueued on `stream`, returns
    without waiting."""
    rc = library().sw_run_device_noalloc(C.byref(cfg), C.c_void_p(state_ptr), C.c_void_p(stream) if stream else None)
    if rc:
        raise NativeError(rc, "sw_run_device_noalloc")


def plan(cfg: Config, cap: int = 4096):
    """sw_plan: (PlanInfo, snapshot times, step count at each snapshot) -- no device needed."""
    info = PlanInfo()
    t = (C.c_double * cap)()
    s = (C.c_int64 * cap)()
    rc = library().sw_plan(C.byref(cfg), C.byref(info), t, s, cap)
    if rc:
        raise NativeError(rc, "sw_plan")
    n = min(info.n_snapshots, cap)
    return info, list(t[:n]), list(s[:n])


def cli_main(problem: int, precision: int, argv: list[str]) -> int:
    """sw_cli_main with argv (argv[0] = program name) -- the bin/*Out programs in-process."""
    arr = (C.c_char_p * (len(argv) + 1))(*[a.encode() for a in argv], None)
    return library().sw_cli_main(problem, precision, len(argv), arr)
