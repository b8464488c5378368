"""Readers of the reference's output files, in Python 3 and without pandas.

* ``Solved`` / ``read_dat``: the .dat solution file (line 1 ``lx nx dx``, then
  rows ``Name t v0 v1 ...``), parsed like ``pyAnalysisTools/result_help.py``
  ``Solved`` (:90-115): times rounded to 7 decimals, the t = 0 rows dropped by
  ``stripInitial``.
* ``Perform``: the timing .txt file (header row, then ``nx tpb us_per_step``
  rows), pivoted nx x tpb like ``pyAnalysisTools/main_help.py`` ``Perform``
  (:14-25).
* ``read_snapshots``: the binary form the programs write when the solution
  path ends in ``.npy`` (a NumPy structured array, record 0 the header); the
  same rows as the .dat, unrounded.  ``read_dat`` and ``Solved`` take either.
"""
from __future__ import annotations

import collections
from pathlib import Path

import numpy as np


ROW_NAMES = {0: ["Temperature"], 1: ["Velocity"], 2: ["Density", "Velocity", "Energy", "Pressure"]}


def read_snapshots(path) -> tuple[list[str], list]:
    """A .npy solution file -> (header fields [lx, nx, dx] as text, rows of
    (name, t, values)), the same shape as read_dat's result.  Values keep the
    run's precision (float32 or float64)."""
    a = np.load(path)
    if a.dtype.names != ("var", "t", "v") or len(a) == 0 or int(a[0]["var"]) != -1:
        raise ValueError("%s is not a swept1d snapshot file" % path)
    h = a[0]
    n, dx, problem = int(h["v"][0]), float(h["v"][1]), int(h["v"][2])
    names = ROW_NAMES[problem]
    rows = [(names[int(r["var"])], float(r["t"]), r["v"]) for r in a[1:]]
    return [repr(float(h["t"])), str(n), repr(dx)], rows


def read_dat(path) -> tuple[list[str], dict]:
    """Return (header fields, rows) with rows = list of (name, t, values)."""
    if str(path).endswith(".npy"):
        return read_snapshots(path)
    with open(path) as f:
        lines = f.read().splitlines()
    head = lines[0].split()
    rows = []
    for ln in lines[1:]:
        parts = ln.split()
        if not parts:
            continue
        rows.append((parts[0], float(parts[1]), np.array([float(v) for v in parts[2:]])))
    return head, rows


class Solved:
    """result_help.Solved: a parsed .dat file."""

    def __init__(self, vFile):
        head, rows = read_dat(vFile)
        self.datafilename = Path(vFile).stem
        self.xGrid = np.linspace(0, float(head[0]), int(head[1]))
        self.numpts = int(head[1])
        self.vals = np.array([r[2] for r in rows])
        self.varNames = np.array([r[0] for r in rows])
        self.tFinal = np.around(np.array([r[1] for r in rows]), decimals=7)
        self.utFinal = np.unique(self.tFinal)
        self.plotTitles = np.unique(self.varNames)
        self.plotname = self.datafilename.split("_")[0]
        self.subpl = "Euler" in self.plotname

    def stripInitial(self) -> dict:
        stripped = collections.defaultdict(dict)
        for i, t in enumerate(self.tFinal):
            if t == 0:
                continue
            stripped[self.varNames[i]][t] = self.vals[i, :]
        return stripped


class Perform:
    """main_help.Perform: a timing file pivoted to {nx: {tpb: us_per_step}}."""

    def __init__(self, dataset):
        with open(dataset) as f:
            lines = [ln.split() for ln in f.read().splitlines() if ln.strip()]
        self.textfile = str(Path(dataset).resolve())
        self.datafilename = Path(dataset).stem
        self.fileLocation = str(Path(dataset).parent)
        self.headers = [h.replace("_", " ") for h in lines[0]]
        self.dataMatrix: dict = collections.defaultdict(dict)
        for row in lines[1:]:
            self.dataMatrix[int(float(row[0]))][int(float(row[1]))] = float(row[2])

    def best(self) -> dict:
        """Best (lowest) us/step per nx and the tpb that gives it."""
        return {nx: min(((v, t) for t, v in d.items())) for nx, d in self.dataMatrix.items()}


TIMING_HEADER = "Num_Spatial_Points\tThreads_per_Block\tTime_per_timestep_(us)\n"


def write_timing_header(path) -> None:
    """The header the reference's drivers write before appending rows
    (sweptPerformanceTest.py:232, quickperform.py:97)."""
    with open(path, "w") as f:
        f.write(TIMING_HEADER)
