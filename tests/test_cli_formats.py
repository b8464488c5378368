"""The drop-in surface on the CPU: the bin/<Problem><Precision>Out argv checks
(which fail before any device work) and the Python 3 ports of the reference's
.dat / timing readers (result_help.Solved, main_help.Perform)."""
import subprocess

import numpy as np
import pytest

PROGS = [p + q + "Out" for p in ("Heat", "KS", "Euler") for q in ("Single", "Double")]


@pytest.fixture(scope="module")
def bins(sw):
    from importlib import import_module
    runner = import_module("1dsweptcuda_gb300.runner")
    paths = {p: runner.ROOT / "bin" / p for p in PROGS}
    missing = [p for p, x in paths.items() if not x.exists()]
    if missing:
        pytest.fail("programs not built: %s" % missing)
    return paths


@pytest.mark.parametrize("prog", PROGS)
def test_usage_message_and_exit(bins, prog, tmp_path):
    r = subprocess.run([str(bins[prog]), "1024", "64"], capture_output=True, text=True)
    assert r.returncode == 255
    assert "The Program takes" in r.stdout


@pytest.mark.parametrize("prog", PROGS)
def test_invalid_sizes_rejected(bins, prog, tmp_path):
    out = tmp_path / "x.dat"
    r = subprocess.run([str(bins[prog]), "1000", "64", "1e-5", "0.01", "1", "1", str(out)], capture_output=True,
                       text=True)
    assert r.returncode == 255
    assert "INVALID NUMERIC INPUT!!" in r.stdout
    r = subprocess.run([str(bins[prog]), "1024", "48", "1e-5", "0.01", "1", "1", str(out)], capture_output=True,
                       text=True)
    assert r.returncode == 255


def test_euler_unstable_dt_rejected(bins, tmp_path):
    r = subprocess.run([str(bins["EulerDoubleOut"]), "1024", "64", "1e-3", "0.1", "1", "1", str(tmp_path / "e.dat")],
                       capture_output=True, text=True)
    assert r.returncode == 255
    assert "is too high" in r.stdout


def test_solved_parser(sw, tmp_path):
    f = tmp_path / "Heat_Double.dat"
    f.write_text("4.095 4 0.001 \nTemperature 0 1 2 3 4 \n Temperature 0.1000000001 5 6 7 8 \n"
                 "Temperature 0.2 9 10 11 12 ")
    s = sw.Solved(f)
    assert s.numpts == 4 and s.plotname == "Heat" and not s.subpl
    assert list(s.tFinal) == [0.0, 0.1, 0.2]
    assert list(s.varNames) == ["Temperature"] * 3
    st = s.stripInitial()
    np.testing.assert_array_equal(st["Temperature"][0.2], [9, 10, 11, 12])
    assert 0.0 not in st["Temperature"]
    np.testing.assert_allclose(s.xGrid, np.linspace(0, 4.095, 4))


def test_solved_parser_euler(sw, tmp_path):
    f = tmp_path / "Euler_Single.dat"
    rows = ["1 2 0.5 "]
    for t in (0, 0.1):
        for n in ("Density", "Velocity", "Energy", "Pressure"):
            rows.append("%s %s 1 2 " % (n, t))
    f.write_text("\n".join(rows) + "\n")
    s = sw.Solved(f)
    assert s.subpl and sorted(s.plotTitles) == ["Density", "Energy", "Pressure", "Velocity"]
    assert set(s.stripInitial()) == {"Density", "Velocity", "Energy", "Pressure"}


def test_perform_parser(sw, tmp_path):
    f = tmp_path / "KS_Double_Swept.txt"
    sw.write_timing_header(f)
    with open(f, "a") as h:
        h.write("1024\t64\t3.5\n1024\t128\t2.5\n2048\t64\t5\n")
    p = sw.Perform(f)
    assert p.headers == ["Num Spatial Points", "Threads per Block", "Time per timestep (us)"]
    assert p.dataMatrix[1024][128] == 2.5
    assert p.best()[1024] == (2.5, 128)


@pytest.mark.parametrize("prog,pid,prec", [("KSDoubleOut", 1, 8), ("HeatSingleOut", 0, 4), ("EulerDoubleOut", 2, 8)])
def test_npy_header_and_initial_rows(sw, oracle, bins, tmp_path, prog, pid, prec):
    """A .npy solution path: the header record and the initial-condition rows
    are written before any device work, so they are checked here with or
    without a GPU (the run itself then fails on a machine without one)."""
    out = tmp_path / "sol.npy"
    subprocess.run([str(bins[prog]), "512", "64", "1e-5", "1e-3", "1e-3", "1", str(out)], capture_output=True,
                   text=True)
    a = np.load(out)
    assert a.dtype.names == ("var", "t", "v")
    assert a["v"].dtype == (np.float64 if prec == 8 else np.float32)
    head, rows = sw.formats.read_snapshots(out)
    ic = oracle.reference_ic(pid, prec, 512)
    n = 510 if pid == 2 else 512
    assert int(head[1]) == n and a["v"].shape[1] == n
    if pid == 2:
        q = ic.reshape(-1, 3)[1:-1]
        assert [r[0] for r in rows[:4]] == ["Density", "Velocity", "Energy", "Pressure"]
        np.testing.assert_array_equal(rows[0][2], q[:, 0])
        np.testing.assert_array_equal(rows[1][2], q[:, 1])          # the IC row holds rho*u, as in the .dat
        np.testing.assert_array_equal(rows[2][2], q[:, 2] / q[:, 0])
    else:
        assert rows[0][0] == ("Temperature" if pid == 0 else "Velocity") and rows[0][1] == 0.0
        np.testing.assert_array_equal(rows[0][2], ic)


def test_snapshot_reader_rejects_other_arrays(sw, tmp_path):
    f = tmp_path / "x.npy"
    np.save(f, np.zeros(4))
    with pytest.raises(ValueError):
        sw.formats.read_snapshots(f)
