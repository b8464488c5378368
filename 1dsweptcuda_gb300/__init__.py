"""swept1d for GB300: swept-rule and classic 1D solvers (Heat, KS, Euler/Sod).

The compute path is ``lib/libswept1d.so`` (hand-written CUDA for sm_103a behind
the C ABI in ``include/swept1d.h``).  This module is its Python binding; it has
no CPU fallback: if the library is missing, importing ``native`` raises.

The package directory name starts with a digit, so import it with
``importlib.import_module("1dsweptcuda_gb300")``.
"""
from __future__ import annotations

from .native import (  # noqa: F401
    ALG_CLASSIC, ALG_SELFTEST, ALG_SWEPT, ALG_VARIANT, BC_DEFAULT, BC_DIRICHLET, BC_MIRROR, BC_PERIODIC,
    EULER, FLAG_HOST_TILE, FLAG_KS_DIVIDE, HEAT, KS, TIME_REFERENCE, TIME_STEPS, Config, Constants, NativeError, Result, Solver, cli_main,
    constants, initial_condition, library, library_path, make_config, plan, validate,
)
from .formats import Perform, Solved, read_dat, read_snapshots, write_timing_header  # noqa: F401
from .runner import runCUDA, binary_path  # noqa: F401

__all__ = [
    "HEAT", "KS", "EULER", "ALG_CLASSIC", "ALG_SWEPT", "ALG_VARIANT", "ALG_SELFTEST",
    "BC_DEFAULT", "BC_MIRROR", "BC_PERIODIC", "BC_DIRICHLET", "TIME_REFERENCE", "TIME_STEPS", "FLAG_KS_DIVIDE", "FLAG_HOST_TILE",
    "Config", "Constants", "Result", "Solver", "NativeError", "make_config", "validate", "constants",
    "initial_condition", "plan", "cli_main", "library", "library_path", "Solved", "Perform", "read_dat",
    "write_timing_header", "runCUDA", "binary_path",
]
