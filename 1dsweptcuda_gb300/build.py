"""Build libswept1d.so (sm_103a) and the bin/<Problem><Precision>Out programs in-tree.

    python 1dsweptcuda_gb300/build.py          # incremental
    python 1dsweptcuda_gb300/build.py --force

Outputs (git-ignored): ``1dsweptcuda_gb300/lib/libswept1d.so`` and
``bin/{Heat,KS,Euler}{Single,Double}Out`` at the repository root.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIBDIR = PKG / "lib"
LIB = LIBDIR / "libswept1d.so"
BIN = ROOT / "bin"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: no contraction anywhere; the stencils also spell every
# operation with a round-to-nearest intrinsic, so they never depend on it.
# -ffp-contract=off for the host compiler: the host tile (host_tile.cu) runs the
# stencils on the CPU, where each operation must round on its own.
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-ffp-contract=off",
                     "-Xptxas", "-warn-spills", "-I", str(INCLUDE)]
# Extra nvcc flags from the environment (e.g. -DSW_EULER_MIN_BLOCKS=3, a tuning macro).
# A change of them is not tracked: rebuild with --force.
NVCC_FLAGS += os.environ.get("SW_NVCC_EXTRA", "").split()
CU_SOURCES = ["k_heat.cu", "k_ks.cu", "k_ks_div.cu", "k_euler.cu", "api.cu", "batch.cu", "noalloc.cu", "closure.cu", "diag.cu",
              "host_tile.cu"]
CPP_SOURCES = ["cli.cpp"]
HEADERS = ["engine.cuh", "stencils.cuh", "persistent.cuh", "sw_internal.h", "ctx.h", "exact_int.h"]
PROGRAMS = [(p, pi, q, qi) for pi, p in enumerate(("Heat", "KS", "Euler")) for q, qi in (("Single", 4), ("Double", 8))]


def _cuda_home() -> Path:
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s" % (" ".join(cmd), r.stdout))


def build(force: bool = False, verbose: bool = False) -> Path:
    OBJ.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    BIN.mkdir(exist_ok=True)
    hdrs = [CSRC / h for h in HEADERS] + [INCLUDE / "swept1d.h"]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        o = OBJ / (src + ".o")
        objs.append(o)
        deps = [CSRC / src] + ([CSRC / "k_ks.cu"] if src == "k_ks_div.cu" else []) + hdrs  # k_ks_div.cu includes k_ks.cu
        if force or _stale(o, deps):
            jobs.append(["nvcc", "-c", str(CSRC / src), "-o", str(o)] + NVCC_FLAGS)
    for src in CPP_SOURCES:
        o = OBJ / (src + ".o")
        objs.append(o)
        if force or _stale(o, [CSRC / src, INCLUDE / "swept1d.h"]):
            # -ffp-contract=off: the .dat writer's derived rows (velocity, energy, pressure)
            # must round like the reference's unfused host code, also where g++ would fuse
            jobs.append(["g++", "-c", str(CSRC / src), "-o", str(o), "-O2", "-std=c++17", "-fPIC",
                         "-ffp-contract=off", "-I", str(INCLUDE)])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            for cmd in jobs:
                if verbose:
                    print(" ".join(cmd))
            list(ex.map(_run, jobs))
    if force or _stale(LIB, objs):
        tmp = LIB.with_name(LIB.name + ".tmp%d" % os.getpid())
        _run(["nvcc", "-shared", "-o", str(tmp)] + [str(o) for o in objs] + ARCH + ["-cudart", "shared"])
        os.replace(tmp, LIB)
    cuda_lib = _cuda_home() / "lib64"
    entry = CSRC / "cli_entry.c"
    for name, pi, qname, qi in PROGRAMS:
        exe = BIN / ("%s%sOut" % (name, qname))
        if force or _stale(exe, [LIB, entry]):
            _run(["gcc", "-O2", "-o", str(exe), str(entry), "-I", str(INCLUDE),
                  "-DSW_PROBLEM=%d" % pi, "-DSW_PRECISION=%d" % qi,
                  "-L", str(LIBDIR), "-lswept1d", "-L", str(cuda_lib),
                  "-Wl,-rpath,$ORIGIN/../1dsweptcuda_gb300/lib"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
