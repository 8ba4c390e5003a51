"""The C ABI library loads and exports every function include/*.h declares
(no kernel is launched here)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"\b(gbba_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_functions():
    names = declared_functions()
    assert "gbba_evaluate_projections" in names
    assert len(names) >= 8


@pytest.mark.parametrize("name", declared_functions())
def test_symbol_exported(name):
    lib = ctypes.CDLL(str(ROOT / "opensfm_gb300" / "libgbba.so"))
    assert hasattr(lib, name), f"{name} declared in include/ but not exported"


def test_num_params_table():
    from opensfm_gb300 import _lib
    L = _lib.lib()
    expected = [3, 9, 3, 8, 12, 16, 1, 4, 6, 5]
    assert [L.gbba_camera_num_params(m) for m in range(10)] == expected
    assert L.gbba_camera_num_params(10) == -1
    assert L.gbba_camera_num_params(-1) == -1
