"""Build recipe for the oracle (TEST INFRASTRUCTURE ONLY).

* ``build_oracle()`` compiles ``oracle.c`` with gcc into
  ``oracle/_build/liboracle.so`` (``-ffp-contract=off``: nothing fused, so the
  oracle keeps the reference's rounding on x86-64 and aarch64 alike).
* ``build_ref()`` compiles ``ref_harness.cu`` against the reference programs
  where they lie, eight times (three problems
  and the KS DIVISE build, x float/double), into
  ``oracle/_ref/libref_<problem>_<f32|f64>.so`` (``libref_ks_div_*`` for DIVISE).  It runs
  only where the reference sources exist; nothing else reads them.

The reference's ``SweptSource`` folder is taken from ``SWEPT1D_REFERENCE_SRC``
when that is set, else from a checkout of the reference named ``reference``
beside this repository's folder (``../reference/SweptSource``).
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
REFERENCE_SRC = Path(os.environ.get("SWEPT1D_REFERENCE_SRC") or HERE.parent.parent / "reference" / "SweptSource")

PROBLEMS = {0: "Heat1D_SweptShared.cu", 1: "KS1D_SweptShared.cu", 2: "Euler1D_SweptShared.cu"}
PROBLEM_NAMES = {0: "heat", 1: "ks", 2: "euler"}


def _newer(target: Path, *sources: Path) -> bool:
    if not target.exists():
        return False
    t = target.stat().st_mtime
    return all(s.stat().st_mtime <= t for s in sources)


def oracle_lib_path() -> Path:
    return BUILD / "liboracle.so"


def build_oracle(force: bool = False) -> Path:
    out = oracle_lib_path()
    srcs = [HERE / "oracle.c", HERE / "oracle.h", HERE / "oracle_impl.h"]
    if not force and _newer(out, *srcs):
        return out
    BUILD.mkdir(exist_ok=True)
    tmp = out.with_suffix(".so.tmp%d" % os.getpid())
    cmd = ["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC",
           "-shared", "-Wall", "-o", str(tmp), str(HERE / "oracle.c"), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, out)
    return out


def reference_available() -> bool:
    return all((REFERENCE_SRC / f).is_file() for f in PROBLEMS.values())


def ref_lib_path(problem: int, prec: int, divide: bool = False) -> Path:
    """divide: the KS DIVISE build's stencil functions (problem 1 only)."""
    name = PROBLEM_NAMES[problem] + ("_div" if divide else "")
    return REF_OUT / ("libref_%s_%s.so" % (name, "f64" if prec == 8 else "f32"))


def _ref_cmd(problem: int, prec: int, out: Path, divide: bool = False) -> list[str]:
    src = REFERENCE_SRC / PROBLEMS[problem]
    cmd = ["nvcc", "-shared", "-Xcompiler", "-fPIC", "-Xcompiler", "-fopenmp", "-Xcompiler", "-ffp-contract=off",
           "-w", "-O2", "-I", str(REFERENCE_SRC), "-DREF_PROBLEM=%d" % problem,
           '-DREF_SRC="%s"' % src, "-o", str(out), str(HERE / "ref_harness.cu")]
    if divide:
        cmd.insert(1, "-DREF_KS_DIVIDE")
    if prec == 8:
        cmd[1:1] = ["-DREAL=double", "-DREALtwo=double2", "-DREALthree=double3", "-DREALfour=double4"]
    return cmd


def build_ref(force: bool = False) -> list[Path]:
    """Compile the reference harness libraries; returns [] when the reference is absent."""
    if not reference_available() or shutil.which("nvcc") is None:
        return []
    REF_OUT.mkdir(exist_ok=True)
    jobs = []
    variants = [(p, False) for p in PROBLEMS] + [(1, True)]  # + the KS DIVISE build
    for problem, divide in variants:
        for prec in (4, 8):
            out = ref_lib_path(problem, prec, divide)
            if not force and _newer(out, HERE / "ref_harness.cu", REFERENCE_SRC / PROBLEMS[problem]):
                continue
            jobs.append((problem, prec, out, divide))

    def run(job):
        problem, prec, out, divide = job
        subprocess.run(_ref_cmd(problem, prec, out, divide), check=True, stdout=subprocess.DEVNULL,
                       stderr=subprocess.PIPE)
        return out

    with ThreadPoolExecutor(max_workers=8) as ex:
        list(ex.map(run, jobs))
    return [ref_lib_path(p, q, d) for p, d in variants for q in (4, 8)]


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_ref(force=True))
