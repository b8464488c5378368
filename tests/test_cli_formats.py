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
