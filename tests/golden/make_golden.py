"""Generate the golden fixtures in this folder from the reference itself.

Run in a checkout where the reference sources exist (SWEPT1D_REFERENCE_SRC, or
by default a checkout named ``reference`` beside this repository's folder,
``../reference/SweptSource``):

    python tests/golden/make_golden.py

It writes

* ``ref_classic.npz`` -- for Heat, KS and Euler in float and double: the
  reference's own initial condition (its ``initFun``) and the state after N
  classic steps computed by the reference's own stencil functions
  (``execFunc``; ``stutterStep``/``finalStep``; ``eulerStutterStep``/
  ``eulerFinalStep``) compiled host-side from the unmodified reference files
  by ``oracle/ref_harness.cu``; for Euler also the reference's ``pressure`` and
  ``energy`` of that state (the .dat writer's derived rows).
* ``ref_ks_divide.npz`` -- KS in float and double at dx = 0.3 (divisors that
  are not powers of two), N classic steps of the reference's DIVISE-build
  stencil functions (KS1D_SweptShared.cu:111-132, built by the harness with
  REF_KS_DIVIDE) and of its default reciprocal build, from one seeded IC.
* ``ks_official.npz`` -- the reference's KS golden run,
  ``SweptSource/Testing/KSDouble_Official.txt`` (nx=1024, dx=0.5, FP64 swept,
  dt=1e-7; Velocity at t = 0, 6, 12, 18, 20), parsed to arrays.

The tests read only these .npz files; they never touch the reference.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from oracle import build as obuild  # noqa: E402
import oracle as O  # noqa: E402

# (problem, nx, dt, nsteps): chosen so every scheme moves visibly.
CASES = [
    (O.HEAT, 256, 0.004, 500),      # Fo = 0.337, insulated ends
    (O.KS, 256, 0.005, 400),        # periodic, t = 2
    (O.EULER, 256, 0.1 / 254, 400),  # dt/dx = 0.1, t = 0.157 (shock well formed)
]
NAMES = {O.HEAT: "heat", O.KS: "ks", O.EULER: "euler"}


def _run_reference(problem, prec, nx, dt, nsteps):
    L = C.CDLL(str(obuild.ref_lib_path(problem, prec)))
    dtype = np.float64 if prec == 8 else np.float32
    assert L.ref_real_size() == prec
    c = O.reference_consts(problem, prec, nx, dt)
    vp = C.c_void_p
    if problem == O.EULER:
        ic = O.reference_ic(problem, prec, nx)  # the reference builds it from bd[] (Euler1D...cu:1179)
        b6 = (C.c_double * 6)(*c.bd)
        L.ref_set(C.c_int64(nx), C.c_double(c.gam), C.c_double(c.mgam), C.c_double(c.dt_dx), b6)
        fin = ic.copy()
        L.ref_classic(vp(fin.ctypes.data), C.c_int64(nx), C.c_int64(nsteps))
        p = np.zeros(nx, dtype)
        e = np.zeros(nx, dtype)
        L.ref_derived(vp(fin.ctypes.data), C.c_int64(nx), vp(p.ctypes.data), vp(e.ctypes.data))
        return ic, fin, {"pressure": p, "energy": e}
    ic = np.zeros(nx, dtype)
    L.ref_ic(C.c_int64(nx), vp(ic.ctypes.data))
    fin = ic.copy()
    if problem == O.HEAT:
        L.ref_classic(vp(fin.ctypes.data), C.c_int64(nx), C.c_double(c.fourier), C.c_double(c.fourier_two),
                      C.c_int64(nsteps))
    else:
        L.ref_classic(vp(fin.ctypes.data), C.c_int64(nx), C.c_double(c.dx_times4), C.c_double(c.dx2),
                      C.c_double(c.dx4), C.c_double(c.dt), C.c_double(c.dt_half), C.c_int64(nsteps))
    return ic, fin, {}


def make_ref_classic():
    libs = obuild.build_ref()
    if not libs:
        raise SystemExit("reference sources not found at %s" % obuild.REFERENCE_SRC)
    out = {}
    for problem, nx, dt, nsteps in CASES:
        for prec in (8, 4):
            key = "%s_f%d" % (NAMES[problem], 8 * prec)
            ic, fin, extra = _run_reference(problem, prec, nx, dt, nsteps)
            out[key + "_ic"] = ic
            out[key + "_final"] = fin
            out[key + "_meta"] = np.array([nx, dt, nsteps], dtype=np.float64)
            for k, v in extra.items():
                out[key + "_" + k] = v
    np.savez_compressed(HERE / "ref_classic.npz", **out)


def make_ref_ks_divide():
    obuild.build_ref()
    nx, dt, dx, nsteps = 256, 5e-4, 0.3, 400
    out = {"meta": np.array([nx, dt, dx, nsteps], dtype=np.float64)}
    for prec in (8, 4):
        dtype = np.float64 if prec == 8 else np.float32
        x = np.arange(nx)
        rng = np.random.default_rng(3)
        ic = (np.cos(2 * np.pi * 5 * x / nx) + 0.1 * rng.standard_normal(nx)).astype(dtype)
        out["f%d_ic" % (8 * prec)] = ic
        for divide in (True, False):
            L = C.CDLL(str(obuild.ref_lib_path(O.KS, prec, divide)))
            assert L.ref_real_size() == prec
            c = O.ks_consts(prec, nx, dt, dx=dx, divide=divide)
            fin = ic.copy()
            L.ref_classic(C.c_void_p(fin.ctypes.data), C.c_int64(nx), C.c_double(c.dx_times4), C.c_double(c.dx2),
                          C.c_double(c.dx4), C.c_double(c.dt), C.c_double(c.dt_half), C.c_int64(nsteps))
            out["f%d_%s" % (8 * prec, "divide" if divide else "multiply")] = fin
    np.savez_compressed(HERE / "ref_ks_divide.npz", **out)


def make_ks_official():
    src = obuild.REFERENCE_SRC / "Testing" / "KSDouble_Official.txt"
    lines = src.read_text().splitlines()
    head = lines[0].split()
    times, rows = [], []
    for ln in lines[1:]:
        parts = ln.split()
        if not parts:
            continue
        assert parts[0] == "Velocity"
        times.append(float(parts[1]))
        rows.append([float(v) for v in parts[2:]])
    np.savez_compressed(HERE / "ks_official.npz", header=np.array([float(h) for h in head]),
                        times=np.array(times), velocity=np.array(rows))


if __name__ == "__main__":
    make_ref_classic()
    make_ref_ks_divide()
    make_ks_official()
    for f in ("ref_classic.npz", "ref_ks_divide.npz", "ks_official.npz"):
        print(f, (HERE / f).stat().st_size, "bytes")
