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


def test_headers_are_plain_c_and_link(tmp_path):
    """Every header compiles as C99 with warnings as errors, and a C program
    linked against libpvglu runs a host-only call through the ABI (symbolic
    analysis of a 3x3 tridiagonal pattern)."""
    import shutil
    import subprocess

    gcc = shutil.which("gcc")
    if gcc is None:
        import pytest

        pytest.skip("no C compiler")
    lib = Path(N.load_library()._name)
    src = tmp_path / "abi.c"
    src.write_text(r"""
#include <stdio.h>
#include "pvglu.h"
#include "pvglu_newton.h"
#include "pvglu_plant.h"
int main(void) {
  const int rowptr[4] = {0, 2, 5, 7};
  const int colidx[7] = {0, 1, 0, 1, 2, 1, 2};
  pvglu_symbolic* s = NULL;
  pvglu_symbolic_info info;
  if (pvglu_symbolic_create(3, rowptr, colidx, NULL, &s) != PVGLU_OK) return 1;
  if (pvglu_symbolic_get_info(s, &info) != PVGLU_OK) return 2;
  printf("%s n=%d nnz_lu=%lld\n", pvglu_version(), info.n, (long long)info.nnz_lu);
  return pvglu_symbolic_destroy(s) == PVGLU_OK && info.n == 3 && info.nnz_lu == 7 ? 0 : 3;
}
""")
    exe = tmp_path / "abi"
    subprocess.run([gcc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I",
                    str(INCLUDE), str(src), "-o", str(exe), "-L", str(lib.parent), "-lpvglu",
                    f"-Wl,-rpath,{lib.parent}"], check=True, timeout=120)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True, timeout=120)
    assert "n=3 nnz_lu=7" in out.stdout


def test_blocks_reject_bad_splits():
    """pvglu_blocks_create checks its split before touching the device: a
    batch that does not divide into the blocks, and zero blocks, are
    PVGLU_ERR_BAD_ARG (1); so are NULL handles to the other blocks calls."""
    import numpy as np

    from phdthesis_albertojimenezruiz_gb300 import FP32, Symbolic

    s = Symbolic(np.array([0, 2, 5, 7]), np.array([0, 1, 0, 1, 2, 1, 2]))
    out = C.c_void_p()
    lib = N.lib()
    for n_scen, parts in ((10, 4), (3, 4), (8, 0), (0, 1)):
        assert lib.pvglu_blocks_create(s.handle, n_scen, parts, FP32, None,
                                       C.byref(out)) == 1, (n_scen, parts)
        assert not out.value
    assert lib.pvglu_blocks_destroy(None) == 1
    assert lib.pvglu_blocks_part(None, 0, C.byref(out)) == 1
    assert lib.pvglu_blocks_step(None, None, None, None, 1e-12, 4, None, 0, None) == 1
    assert lib.pvglu_blocks_join(None, None) == 1
