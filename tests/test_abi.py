"""C-ABI surface (CPU): the library loads and exports every function that
include/*.h declares, and the Python binding declares no symbol the headers
do not have."""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

from phdthesis_albertojimenezruiz_gb300 import _native as N

INCLUDE = Path(__file__).resolve().parent.parent / "include"


def declared_functions() -> set[str]:
    names = set()
    for h in INCLUDE.glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"\b(pvglu_\w+)\s*\(", text):
            # skip typedef'd struct names used as types (followed by '*')
            names.add(m.group(1))
    return names


def test_headers_declare_functions():
    names = declared_functions()
    assert "pvglu_refactor" in names and "pvglu_symbolic_create" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(str(N._LIB_PATH))
    missing = [n for n in sorted(declared_functions()) if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_matches_headers():
    assert set(N.exported_symbols()) <= declared_functions()


def test_version_and_error_string():
    assert N.lib().pvglu_version().startswith(b"pvglu")
    assert N.lib().pvglu_last_error() is not None
