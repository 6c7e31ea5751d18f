"""The C ABI: libtt.so loads and exports every function include/*.h declares; error reporting."""
import ctypes as C
import re
from pathlib import Path

import pytest

from trenchanttracer_gb300 import BVHCompact, TTError, _lib

ROOT = Path(__file__).resolve().parents[1]


def declared_functions() -> list[str]:
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"\b(tt_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    assert "tt_trace" in names and "tt_bvh_build" in names and len(names) >= 15


@pytest.mark.parametrize("name", declared_functions())
def test_library_exports(name):
    lib = C.CDLL(str(_lib.LIB_PATH))
    assert hasattr(lib, name), f"libtt.so does not export {name}"


def test_python_binding_covers_header():
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_version_and_error_reporting(tmp_path):
    assert b"sm_103a" in _lib.lib().tt_version()
    with pytest.raises(TTError) as e:
        BVHCompact.load(tmp_path / "missing.cache")
    assert e.value.status == 2  # TT_ERR_IO
    assert "missing.cache" in str(e.value)


def test_null_arguments_are_rejected():
    lib = _lib.lib()
    assert lib.tt_bvh_build(None, 1e-5, 1, 8, 0, None) == 1
    assert lib.tt_trace(None, None, 0, None, 1, None) == 1
    assert lib.tt_bvh_upload(None, None) == 1
