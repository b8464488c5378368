import importlib
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the native library's kernels)")
    config.addinivalue_line("markers", "slow: long-running case")


@pytest.fixture(scope="session")
def sw():
    """The product package (native CUDA library binding)."""
    return importlib.import_module("1dsweptcuda_gb300")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    return O


@pytest.fixture(scope="session")
def solver(sw):
    s = sw.Solver(0)
    yield s
    s.close()


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return {
        "ref": np.load(ROOT / "tests" / "golden" / "ref_classic.npz"),
        "ks": np.load(ROOT / "tests" / "golden" / "ks_official.npz"),
        "ks_divide": np.load(ROOT / "tests" / "golden" / "ref_ks_divide.npz"),
    }
