"""CPU oracle for the swept 1D solvers -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py``
import this package, to check results.  The product path (the CUDA library in
``1dsweptcuda_gb300``) never imports or calls it.

``liboracle.so`` (``oracle.c``) restates the reference's classic schemes in its
own operation order (see ``oracle.h`` for file:line citations); ``exact.py``
holds the analytic solutions the reference's tests compare against.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

HEAT, KS, EULER = 0, 1, 2
BC_MIRROR, BC_PERIODIC, BC_DIRICHLET = 1, 2, 3
RADIUS = {HEAT: 1, KS: 2, EULER: 2}
SUBSTEPS = {HEAT: 1, KS: 2, EULER: 2}
COMPONENTS = {HEAT: 1, KS: 1, EULER: 3}


class Consts(C.Structure):
    _fields_ = [
        ("problem", C.c_int), ("bc", C.c_int), ("nx", C.c_int64),
        ("fourier", C.c_double), ("fourier_two", C.c_double),
        ("dx_times4", C.c_double), ("dx2", C.c_double), ("dx4", C.c_double),
        ("dt", C.c_double), ("dt_half", C.c_double),
        ("gam", C.c_double), ("mgam", C.c_double), ("dt_dx", C.c_double),
        ("bd", C.c_double * 6), ("divide", C.c_int),
    ]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "bd"}
        d["bd"] = list(self.bd)
        return d


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = C.CDLL(str(path))
        P = C.POINTER(Consts)
        for sfx, ct in (("f64", C.c_double), ("f32", C.c_float)):
            for name, extra in (("or_classic_", [C.c_int64]), ("or_classic_omp_", [C.c_int64, C.c_int])):
                f = getattr(L, name + sfx)
                f.argtypes = [P, C.c_void_p] + extra
                f.restype = C.c_int
            f = getattr(L, "or_swept_" + sfx)
            f.argtypes = [P, C.c_void_p, C.c_int, C.c_int64]
            f.restype = C.c_int64
            f = getattr(L, "or_euler_pressure_" + sfx)
            f.argtypes = [P, C.c_void_p]
            f.restype = C.c_double
        L.or_reference_consts.argtypes = [C.c_int, C.c_int, C.c_int64, C.c_double, P]
        L.or_reference_consts.restype = C.c_int
        L.or_reference_ic.argtypes = [C.c_int, C.c_int, C.c_int64, C.c_void_p]
        L.or_reference_ic.restype = C.c_int
        L.or_openmp_max_threads.restype = C.c_int
        _lib = L
    return _lib


def _dtype(prec: int):
    return np.float64 if prec == 8 else np.float32


def _sfx(arr: np.ndarray) -> str:
    if arr.dtype == np.float64:
        return "f64"
    if arr.dtype == np.float32:
        return "f32"
    raise TypeError("oracle state must be float32 or float64, got %s" % arr.dtype)


def reference_consts(problem: int, prec: int, nx: int, dt: float) -> Consts:
    """The constants the reference's main() derives for a CLI run (REAL-rounded)."""
    c = Consts()
    if lib().or_reference_consts(problem, prec, nx, dt, C.byref(c)):
        raise ValueError("bad constants request")
    return c


def ks_consts(prec: int, nx: int, dt: float, dx: float = 0.5, divide: bool = False) -> Consts:
    """KS constants at a given dx, rounded through REAL as main() rounds them:
    the reciprocals 1/(4dx), 1/dx^2, 1/dx^4 (KS1D_SweptShared.cu:917-926), or
    with ``divide`` the DIVISE build's divisors 4dx, dx^2, dx^4 (:904-914)."""
    c = reference_consts(KS, prec, nx, dt)
    R = np.float64 if prec == 8 else np.float32
    d = R(dx)
    if divide:
        c4, d2, d4 = R(4) * d, d * d, d * d * d * d
    else:
        c4, d2, d4 = R(1) / (R(4) * d), R(1) / (d * d), R(1) / (d * d * d * d)
    c.dx_times4, c.dx2, c.dx4 = float(c4), float(d2), float(d4)
    c.divide = 1 if divide else 0
    return c


def reference_ic(problem: int, prec: int, nx: int) -> np.ndarray:
    """The reference's initial condition (Heat parabola, KS cosine, Sod tube)."""
    out = np.zeros(nx * COMPONENTS[problem], dtype=_dtype(prec))
    if lib().or_reference_ic(problem, prec, nx, out.ctypes.data):
        raise ValueError("bad IC request")
    return out


def classic(c: Consts, u: np.ndarray, nsteps: int, threads: int | None = None) -> np.ndarray:
    """Advance a copy of ``u`` by ``nsteps`` classic time steps (threads: OpenMP)."""
    u = np.ascontiguousarray(u).copy()
    L = lib()
    if threads is None:
        rc = getattr(L, "or_classic_" + _sfx(u))(C.byref(c), u.ctypes.data, nsteps)
    else:
        rc = getattr(L, "or_classic_omp_" + _sfx(u))(C.byref(c), u.ctypes.data, nsteps, threads)
    if rc:
        raise RuntimeError("oracle classic failed: %d" % rc)
    return u


def swept(c: Consts, u: np.ndarray, tpb: int, n_diamonds: int) -> tuple[np.ndarray, int]:
    """CPU model of the swept decomposition; returns (state, time steps advanced)."""
    u = np.ascontiguousarray(u).copy()
    n = getattr(lib(), "or_swept_" + _sfx(u))(C.byref(c), u.ctypes.data, tpb, n_diamonds)
    if n < 0:
        raise ValueError("bad swept request: %d" % n)
    return u, int(n)


def euler_pressure(c: Consts, q3: np.ndarray) -> np.ndarray:
    q3 = np.ascontiguousarray(q3).reshape(-1, 3)
    f = getattr(lib(), "or_euler_pressure_" + _sfx(q3))
    out = np.empty(len(q3), dtype=q3.dtype)
    for i in range(len(q3)):
        out[i] = f(C.byref(c), q3[i].ctypes.data)
    return out


def openmp_threads() -> int:
    return int(lib().or_openmp_max_threads())


def make_consts(problem: int, nx: int, prec: int = 8, bc: int | None = None, **kw) -> Consts:
    """Constants for a non-CLI case: start from the reference values for dt
    and override fields by keyword (e.g. fourier=..., bc=BC_PERIODIC)."""
    dt = kw.pop("dt", 1e-3 if problem != EULER else 1e-6)
    c = reference_consts(problem, prec, nx, dt)
    if bc is not None:
        c.bc = bc
    for k, v in kw.items():
        if k == "bd":
            for i in range(6):
                c.bd[i] = v[i]
        else:
            setattr(c, k, v)
    return c


def quantum_steps(problem: int, tpb: int) -> int:
    """Time steps per swept half-cycle (one diamond): tpb / (2 R S)."""
    return tpb // (2 * RADIUS[problem] * SUBSTEPS[problem])


