"""The C ABI on the CPU: the library loads, exports every function the header
declares, agrees with the header's struct layouts, validates like the
reference's main(), derives its constants and initial conditions exactly, and
plans runs with the reference wrappers' time bookkeeping.  No kernel runs."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import schedule

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "swept1d.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sw_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_function(sw):
    lib = sw.library()
    names = declared_functions()
    assert "sw_run" in names and "sw_cli_main" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", str(sw.library_path())], capture_output=True, text=True)
    if out.returncode == 0:
        exported = set(re.findall(r" T (sw_\w+)", out.stdout))
        assert set(names) <= exported, set(names) - exported


def test_python_binding_lists_the_header(sw):
    from importlib import import_module
    native = import_module("1dsweptcuda_gb300.native")
    assert sorted(native.EXPORTED) == declared_functions()


def test_struct_layouts_match_header(sw, tmp_path):
    """sizeof/offsetof of the ABI structs from a C compile of the header equal the ctypes mirrors."""
    from importlib import import_module
    native = import_module("1dsweptcuda_gb300.native")
    src = tmp_path / "l.c"
    fields = {"sw_config": native.Config, "sw_constants": native.Constants, "sw_result": native.Result,
              "sw_plan_info": native.PlanInfo, "sw_tuning": native.Tuning, "sw_adaptive_info": native.AdaptiveInfo}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "swept1d.h"', "int main(void){"]
    for cname, py in fields.items():
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in py._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines.append("return 0;}")
    src.write_text("\n".join(lines))
    exe = tmp_path / "l"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), "-o", str(exe), str(src)], check=True)
    got = dict(ln.split() for ln in subprocess.run([str(exe)], capture_output=True, text=True).stdout.splitlines())
    for cname, py in fields.items():
        assert int(got[cname]) == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert int(got["%s.%s" % (cname, f)]) == getattr(py, f).offset, (cname, f)


def test_enum_values_match_header(sw, tmp_path):
    """The Python binding's enum constants equal the header's."""
    from importlib import import_module
    native = import_module("1dsweptcuda_gb300.native")
    names = {"SW_HEAT": native.HEAT, "SW_KS": native.KS, "SW_EULER": native.EULER,
             "SW_ALG_CLASSIC": native.ALG_CLASSIC, "SW_ALG_SWEPT": native.ALG_SWEPT,
             "SW_ALG_VARIANT": native.ALG_VARIANT, "SW_ALG_SELFTEST": native.ALG_SELFTEST,
             "SW_BC_DEFAULT": native.BC_DEFAULT, "SW_BC_MIRROR": native.BC_MIRROR,
             "SW_BC_PERIODIC": native.BC_PERIODIC, "SW_BC_DIRICHLET": native.BC_DIRICHLET,
             "SW_TIME_REFERENCE": native.TIME_REFERENCE, "SW_TIME_STEPS": native.TIME_STEPS,
             "SW_FLAG_KS_DIVIDE": native.FLAG_KS_DIVIDE, "SW_FLAG_HOST_TILE": native.FLAG_HOST_TILE}
    src = tmp_path / "e.c"
    src.write_text("\n".join(['#include <stdio.h>', '#include "swept1d.h"', "int main(void){"] +
                              ['printf("%s %%d\\n", (int)%s);' % (n, n) for n in names] + ["return 0;}"]))
    exe = tmp_path / "e"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), "-o", str(exe), str(src)], check=True)
    got = dict(ln.split() for ln in subprocess.run([str(exe)], capture_output=True, text=True).stdout.splitlines())
    assert {k: int(v) for k, v in got.items()} == names


def test_strerror_and_version(sw):
    lib = sw.library()
    assert lib.sw_abi_version() == 1
    for code in range(0, -11, -1):
        assert lib.sw_strerror(code)
    assert lib.sw_strerror(-999) == b"unknown error"


@pytest.mark.parametrize("problem", [0, 1, 2])
@pytest.mark.parametrize("prec", [4, 8])
def test_constants_and_ic_match_oracle(sw, oracle, problem, prec):
    for nx, dt in ((256, 0.001), (4096, 1e-5), (1 << 20, 0.005)):
        if problem == 2:
            dt = min(dt, 0.2 / nx)
        cfg = sw.make_config(problem, prec, nx=nx, tpb=256, dt=dt)
        k = sw.constants(cfg)
        c = oracle.reference_consts(problem, prec, nx, dt)
        for f in ("fourier", "fourier_two", "dx_times4", "dx2", "dx4", "dt", "dt_half", "gam", "mgam", "dt_dx"):
            assert getattr(k, f) == getattr(c, f), f
        assert list(k.bd) == list(c.bd)
        if nx <= 4096:
            np.testing.assert_array_equal(sw.initial_condition(cfg), oracle.reference_ic(problem, prec, nx))


def test_validation_codes(sw):
    ok = dict(nx=1024, tpb=64, dt=0.001)
    assert sw.validate(sw.make_config(1, 8, **ok)) == 0
    assert sw.validate(sw.make_config(1, 8, nx=1000, tpb=64, dt=0.001)) == -2     # tpb does not divide nx
    assert sw.validate(sw.make_config(1, 8, nx=1024, tpb=48, dt=0.001)) == -2     # tpb not a multiple of 32
    assert sw.validate(sw.make_config(1, 8, nx=1024, tpb=2048, dt=0.001)) == -2   # tpb above 1024
    assert sw.validate(sw.make_config(1, 8, nx=32, tpb=64, dt=0.001)) == -2       # nx below tpb
    assert sw.validate(sw.make_config(2, 8, nx=1024, tpb=64, dt=0.3 / 1022)) == -3  # Euler dt/dx > 0.21
    assert sw.validate(sw.make_config(2, 8, nx=1024, tpb=64, dt=0.2 / 1022)) == 0
    assert sw.validate(sw.make_config(1, 8, nx=1024, tpb=64, dt=0.001, bc=sw.BC_MIRROR)) == -1  # KS is periodic
    assert sw.validate(sw.make_config(0, 8, nx=1024, tpb=64, dt=0.001, bc=sw.BC_PERIODIC)) == 0
    assert sw.validate(sw.make_config(0, 8, nx=1024, tpb=64, dt=0.001, alg=3)) == -1  # self-test is KS only
    assert sw.validate(sw.make_config(1, 8, nx=1024, tpb=64, dt=-1.0)) == -1
    bad = sw.make_config(1, 8, **ok)
    bad.precision = 2
    assert sw.validate(bad) == -1


def test_custom_physics(sw):
    """Non-reference constants: Heat diffusivity/dx, Euler gamma and states."""
    k = sw.constants(sw.make_config(0, 8, nx=1024, tpb=64, dt=1e-3, alpha=1e-4, dx=0.01))
    assert k.fourier == 1e-4 * 1e-3 / (0.01 * 0.01)
    k = sw.constants(sw.make_config(2, 8, nx=1024, tpb=64, dt=1e-5, gamma=5 / 3, left=(2.0, 0.5, 3.0),
                                    right=(1.0, 0.0, 1.0)))
    assert k.mgam == 5 / 3 - 1
    assert k.bd[0] == 2.0 and k.bd[1] == 1.0 and abs(k.bd[2] - (3.0 / (5 / 3 - 1) + 0.5 * 2.0 * 0.25)) < 1e-12


CASES = [
    # problem, prec, alg, tpb, dt, tf, freq
    (0, 8, 0, 128, 1e-5, 0.05, 0.02), (0, 8, 1, 128, 1e-5, 0.05, 0.02), (0, 8, 2, 128, 1e-5, 0.05, 0.02),
    (0, 4, 1, 64, 1e-4, 1.0, 0.3), (0, 8, 0, 64, 1e-4, 1.0, 0.3),
    (1, 8, 0, 128, 1e-3, 2.0, 0.5), (1, 8, 1, 128, 1e-3, 2.0, 0.5), (1, 8, 2, 256, 1e-3, 2.0, 0.5),
    (1, 4, 0, 64, 3e-3, 2.0, 0.7), (1, 4, 1, 64, 3e-3, 2.0, 0.7), (1, 4, 2, 64, 3e-3, 2.0, 0.7),
    (2, 8, 0, 128, 1e-5, 0.02, 0.006), (2, 8, 1, 128, 1e-5, 0.02, 0.006), (2, 4, 2, 64, 1e-5, 0.02, 0.006),
    (1, 8, 1, 1024, 5e-3, 200.0, 50.0), (1, 8, 0, 256, 5e-3, 200.0, 1000.0),
]


@pytest.mark.parametrize("case", CASES)
def test_plan_follows_reference_bookkeeping(sw, case):
    """sw_plan (the library's loop planner) == a direct restatement of the
    reference wrappers' loops: final t_eq, steps advanced, snapshot times/steps."""
    problem, prec, alg, tpb, dt, tf, freq = case
    nx = 4 * tpb if problem != 2 else 4 * tpb
    if problem == 2:
        dt = min(dt, 0.2 / (nx - 2))
    cfg = sw.make_config(problem, prec, alg=alg, nx=nx, tpb=tpb, dt=dt, tf=tf, freq=freq)
    info, ts, steps = sw.plan(cfg)
    t_final, n, snaps = schedule.reference_schedule(problem, prec, alg, tpb, dt, tf, freq)
    assert info.t_final == t_final
    assert info.n_steps == n
    assert info.n_snapshots == len(snaps)
    assert ts == [s[0] for s in snaps]
    assert steps == [s[1] for s in snaps]


def test_plan_exact_steps(sw):
    """SW_TIME_STEPS: exactly n steps; swept finishes the remainder classically."""
    for alg in (0, 1, 2):
        cfg = sw.make_config(1, 8, alg=alg, nx=4096, tpb=256, dt=0.005, time_mode=sw.TIME_STEPS, n_steps=1000)
        info, _, _ = sw.plan(cfg)
        assert info.n_steps == 1000 and abs(info.t_final - 5.0) < 1e-12
    cfg = sw.make_config(1, 8, alg=1, nx=1 << 20, tpb=256, dt=0.005, time_mode=sw.TIME_STEPS, n_steps=40000)
    info, _, _ = sw.plan(cfg)
    assert info.launches == 40000 // 32 + 1 and info.tile == 256  # up + 1249 diamonds + down


def test_ensemble_generator():
    """The ensemble workload: log-uniform nx in 2^10..2^16 (mean ~18.6k), 8 modes with N(0,1)/k amplitudes."""
    from importlib import import_module
    ens = import_module("1dsweptcuda_gb300.ensemble")
    nx, u = ens.make_ensemble(n_domains=4096)
    e = np.log2(nx).astype(int)
    assert e.min() == 10 and e.max() == 16 and set(np.unique(e)) == set(range(10, 17))
    assert 17000 < nx.mean() < 20000
    assert u.size == nx.sum() and np.isfinite(u).all()
    parts = ens.split(u, nx)
    assert [len(p) for p in parts] == list(nx)
    # each domain is a trigonometric polynomial of its own period: zero mean
    assert max(abs(float(p.mean())) for p in parts[:50]) < 1e-9
    nx2, u2 = ens.make_ensemble(n_domains=4096)
    assert (nx2 == nx).all() and np.array_equal(u2, u)   # seeded


def test_host_tile_flag_rules(sw):
    """SW_FLAG_HOST_TILE: alg 1 for any problem, alg 2 for Heat and Euler (the
    reference's hybrid), never with the dividing KS build or classic."""
    ok = [(0, 1), (0, 2), (2, 1), (2, 2), (1, 1)]
    bad = [(1, 2), (0, 0), (1, 0)]
    for problem, alg in ok + bad:
        dt = 1e-5 if problem == 2 else 1e-3
        cfg = sw.make_config(problem, 8, alg=alg, nx=1024, tpb=64, dt=dt, flags=sw.FLAG_HOST_TILE)
        assert (sw.validate(cfg) == 0) == ((problem, alg) in ok), (problem, alg)
    ks = sw.make_config(1, 8, alg=1, nx=1024, tpb=64, dt=1e-3, flags=sw.FLAG_HOST_TILE | sw.FLAG_KS_DIVIDE)
    assert sw.validate(ks) == -1
