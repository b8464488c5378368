"""runCUDA: the reference's program runner (pyAnalysisTools/main_help.py:47-66)
in Python 3, pointed at this project's bin/<Problem><Precision>Out programs."""
from __future__ import annotations

import shlex
import subprocess as sp
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def binary_path(problem: str, precision: str = "Double") -> Path:
    """bin/<Problem><Precision>Out, e.g. binary_path("KS", "Double")."""
    return ROOT / "bin" / ("%s%sOut" % (problem, precision))


def _as_list(v):
    return v if isinstance(v, list) else [v]


def runCUDA(Prog, divisions, threadsPerBlock, timeStep, finishTime, frequency, decomp, varfile="temp.dat",
            timefile="", quiet=False):
    """Run Prog for every (tpb, nx) pair with the reference's argv order:
    nx tpb dt tf freq alg varfile [timefile].  Returns the exit codes."""
    codes = []
    for tpb in _as_list(threadsPerBlock):
        for dvs in _as_list(divisions):
            cmd = "%s %s %s %s %s %s %s %s %s" % (Prog, dvs, tpb, timeStep, finishTime, frequency, decomp,
                                                  varfile, timefile)
            out = sp.DEVNULL if quiet else None
            codes.append(sp.call(shlex.split(cmd), stdout=out))
    return codes
