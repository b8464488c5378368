"""Every committed Python entry point at least compiles (CPU)."""
import py_compile
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
SCRIPTS = sorted([ROOT / "bench.py", ROOT / "__graft_entry__.py"] + list((ROOT / "1dsweptcuda_gb300").glob("*.py"))
                 + list((ROOT / "oracle").glob("*.py")) + list((ROOT / "tests" / "golden").glob("*.py")))


@pytest.mark.parametrize("path", SCRIPTS, ids=lambda p: str(p.relative_to(ROOT)))
def test_compiles(path, tmp_path):
    py_compile.compile(str(path), cfile=str(tmp_path / "x.pyc"), doraise=True)
