"""The bin/<Problem><Precision>Out programs on a GPU: argv, .dat rows, the
timing file, the consistency procedure of the reference's testProcedure.py and
the KS self-test (alg 3)."""
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PID = {"Heat": 0, "KS": 1, "Euler": 2}


def _bin(sw, name):
    from importlib import import_module
    return import_module("1dsweptcuda_gb300.runner").ROOT / "bin" / name


def _run(path, args, ok=True):
    r = subprocess.run([str(path)] + [str(a) for a in args], capture_output=True, text=True, timeout=600)
    if ok:
        assert r.returncode == 0, r.stdout + r.stderr
    return r


def _fmt(v):
    # what an ostream with precision(10) prints for the value (float promoted to double)
    return "%.10g" % float(v)


@pytest.mark.parametrize("prec", ["Single", "Double"])
@pytest.mark.parametrize("prob", ["Heat", "KS", "Euler"])
@pytest.mark.parametrize("alg", [0, 1, 2])
def test_dat_rows_equal_oracle_text(sw, oracle, tmp_path, prob, prec, alg):
    """Every number the program writes equals the oracle's value printed the same way."""
    p = PID[prob]
    nx, tpb = 512, 64
    dt = {0: 0.004, 1: 0.005, 2: 0.1 / 510}[p]
    q = tpb // (2 * oracle.RADIUS[p] * oracle.SUBSTEPS[p])
    tf, freq = 24 * q * dt, 9 * q * dt
    out = tmp_path / ("%s_%s.dat" % (prob, prec))
    _run(_bin(sw, prob + prec + "Out"), [nx, tpb, repr(dt), repr(tf), repr(freq), alg, out])
    s = sw.Solved(out)
    bytes_ = 8 if prec == "Double" else 4
    c = oracle.reference_consts(p, bytes_, nx, dt)
    ic = oracle.reference_ic(p, bytes_, nx)
    cfg = sw.make_config(p, bytes_, alg=alg, nx=nx, tpb=tpb, dt=dt, tf=tf, freq=freq)
    info, ts, steps = sw.plan(cfg)
    lines = out.read_text().splitlines()
    body = [ln.split() for ln in lines[1:] if ln.strip()]
    times = [0.0] + ts + [info.t_final]
    nsteps = [0] + steps + [info.n_steps]
    per = 4 if p == 2 else 1
    assert len(body) == per * len(times)
    for k, (t, n) in enumerate(zip(times, nsteps)):
        u = oracle.classic(c, ic, n)
        if p == 2:
            q3 = u.reshape(-1, 3)[1:-1].astype(np.float64)
            dtp = np.float32 if bytes_ == 4 else np.float64
            qq = u.reshape(-1, 3)[1:-1]
            rho, m, E = qq[:, 0], qq[:, 1], qq[:, 2]
            vel = (m / rho).astype(dtp) if k else m
            half = dtp(0.5)
            uu = (m / rho).astype(dtp)
            ener = (E / rho - half * uu * uu).astype(dtp) if k else (E / rho).astype(dtp)
            pres = oracle.euler_pressure(c, u)[1:-1]
            want_rows = [("Density", rho), ("Velocity", vel), ("Energy", ener), ("Pressure", pres)]
            for j, (name, vals) in enumerate(want_rows):
                row = body[per * k + j]
                assert row[0] == name
                assert row[1] == _fmt(t) if k else row[1] == "0"
                assert row[2:] == [_fmt(v) for v in vals], (name, t)
        else:
            row = body[k]
            assert row[0] == ("Temperature" if p == 0 else "Velocity")
            assert row[2:] == [_fmt(v) for v in u], (prob, t)
    del s


def test_timing_file_rows(sw, tmp_path):
    tf = tmp_path / "KS_Double_Swept.txt"
    sw.write_timing_header(tf)
    for tpb in (64, 128):
        _run(_bin(sw, "KSDoubleOut"), [4096, tpb, 0.005, 1.0, 2.0, 1, tmp_path / "a.dat", tf])
    p = sw.Perform(tf)
    assert set(p.dataMatrix[4096]) == {64, 128}
    assert all(v > 0 for v in p.dataMatrix[4096].values())


@pytest.mark.parametrize("prob,tf", [("Heat", 0.5), ("KS", 1.0), ("Euler", 0.02)])
def test_consistency_procedure(sw, tmp_path, prob, tf):
    """testProcedure.consistency (:106-122): swept, variant, classic at nx=4096,
    tpb=128, dt=1e-5, each run to the previous run's final time; the final rows
    must agree with RMSE 0 (the reference recorded 0.000e+00 on every variable)."""
    prog = _bin(sw, prob + "DoubleOut")
    vfile = tmp_path / (prob + "_temp.dat")
    finals = []
    for alg in (1, 2, 0):
        _run(prog, [4096, 128, 1e-5, repr(tf), repr(tf * 2.0), alg, vfile])
        s = sw.Solved(vfile)
        last = s.tFinal[-1]
        finals.append({n: s.vals[i] for i, n in enumerate(s.varNames) if s.tFinal[i] == last})
        tf = float(open(vfile).read().splitlines()[-1].split()[1])
    for alg_rows in finals[:2]:
        for name, vals in alg_rows.items():
            rmse = float(np.sqrt(np.mean((vals - finals[2][name]) ** 2)))
            assert rmse == 0.0, (prob, name, rmse)


def test_ks_selftest(sw, tmp_path):
    """alg 3: variant kernels vs shared kernels, EQUAL! on every stage, exit -1."""
    r = _run(_bin(sw, "KSDoubleOut"), [1024, 64, 1e-5, 0.01, 1, 3, tmp_path / "k.dat"], ok=False)
    assert r.returncode == 255
    assert r.stdout.count("EQUAL!") == 3 and "NOT EQUAL" not in r.stdout, r.stdout


@pytest.mark.parametrize("prec", ["Single", "Double"])
@pytest.mark.parametrize("prob", ["Heat", "KS", "Euler"])
def test_npy_rows_equal_dat_rows(sw, oracle, tmp_path, prob, prec):
    """The .npy solution holds the .dat's rows: same names and times, and every
    value printed at precision 10 is the .dat's token; the final row is the
    oracle's classic state itself, unrounded."""
    p = PID[prob]
    nx, tpb = 512, 64
    dt = {0: 0.004, 1: 0.005, 2: 0.1 / 510}[p]
    q = tpb // (2 * oracle.RADIUS[p] * oracle.SUBSTEPS[p])
    tf, freq = 24 * q * dt, 9 * q * dt
    dat, npy = tmp_path / "s.dat", tmp_path / "s.npy"
    args = [nx, tpb, repr(dt), repr(tf), repr(freq), 1]
    _run(_bin(sw, prob + prec + "Out"), args + [dat])
    _run(_bin(sw, prob + prec + "Out"), args + [npy])
    hd, rd = sw.read_dat(dat)
    hn, rn = sw.read_dat(npy)
    assert int(hn[1]) == int(hd[1]) and len(rn) == len(rd)
    assert abs(float(hn[0]) - float(hd[0])) <= 1e-9 * float(hd[0])
    text_rows = [ln.split() for ln in dat.read_text().splitlines()[1:] if ln.strip()]
    for (name_d, t_d, _), (name_n, t_n, v_n), tokens in zip(rd, rn, text_rows):
        assert name_n == name_d
        assert abs(t_n - t_d) <= 1e-9 * max(1.0, abs(t_d))
        assert tokens[2:] == [_fmt(v) for v in v_n], (prob, prec, t_n)
    bytes_ = 8 if prec == "Double" else 4
    cfg = sw.make_config(p, bytes_, alg=1, nx=nx, tpb=tpb, dt=dt, tf=tf, freq=freq)
    info, _, _ = sw.plan(cfg)
    fin = oracle.classic(oracle.reference_consts(p, bytes_, nx, dt), oracle.reference_ic(p, bytes_, nx), info.n_steps)
    if p == 2:
        np.testing.assert_array_equal(rn[-4][2], fin.reshape(-1, 3)[1:-1, 0])
    else:
        np.testing.assert_array_equal(rn[-1][2], fin)


def test_ks_divide_environment(sw, tmp_path):
    """SWEPT1D_KS_DIVIDE=1 selects the DIVISE build's division form; at the
    programs' dx = 0.5 it writes the same file as the reciprocal form."""
    import os
    files = []
    for env in ("0", "1"):
        out = tmp_path / ("ks_%s.dat" % env)
        r = subprocess.run([str(_bin(sw, "KSDoubleOut")), "1024", "128", "0.005", "2", "0.5", "1", str(out)],
                           capture_output=True, text=True, timeout=600, env=dict(os.environ, SWEPT1D_KS_DIVIDE=env))
        assert r.returncode == 0, r.stdout + r.stderr
        files.append(out.read_bytes())
    assert files[0] == files[1]
