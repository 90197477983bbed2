"""The C-ABI library loads and exports every entry point ``include/fvgb.h`` declares (no GPU)."""
from __future__ import annotations

import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    with open(os.path.join(ROOT, "include", "fvgb.h")) as fh:
        text = fh.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fv_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def library():
    from aquaflux_gb300 import _lib

    if not os.path.exists(_lib.LIB_PATH):
        from aquaflux_gb300 import build

        build.build_library()
    return ctypes.CDLL(_lib.LIB_PATH)


def test_every_declared_symbol_is_exported(library):
    names = _declared()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(library, n)]
    assert not missing, missing


def test_binding_table_covers_the_header():
    from aquaflux_gb300 import _lib

    assert sorted(_lib.SIGNATURES) == _declared()


def test_version_and_error_string(library):
    library.fv_version.restype = ctypes.c_char_p
    assert b"sm_103a" in library.fv_version()
    library.fv_last_error.restype = ctypes.c_char_p
    assert isinstance(library.fv_last_error(), bytes)


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    from aquaflux_gb300 import _lib

    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "absent.so"))
    monkeypatch.setattr(_lib, "_lib", None)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _lib.lib()
