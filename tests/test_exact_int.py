"""The FP64 products the kernels form on the integer pipe (csrc/exact_int.h:
6 * x and x * 2^k) give the bits of the FP64 multiply: the same header,
compiled for the host, against the host's IEEE multiply on random operands,
constructed rounding ties and special values."""
import shutil
import subprocess
from pathlib import Path

import pytest

HERE = Path(__file__).resolve().parent


def test_integer_pipe_products_round_like_the_multiply(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no host C++ compiler")
    exe = tmp_path / "exact_int_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-o", str(exe), str(HERE / "exact_int_check.cpp")], check=True)
    out = subprocess.run([str(exe), "400000"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "differ 0" in out.stdout
