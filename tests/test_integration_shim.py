"""The drop-in shim of INTEGRATION.md (the C++ file a maintainer links into the
reference's driver in place of factorize_electrical_system_CUDA.cu and
triangular_substitution.cu) compiles against the reference's own headers and
ours (CPU; skipped where the reference sources are absent)."""
from __future__ import annotations

import re
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_shim_compiles_against_reference_headers(tmp_path):
    from oracle import oracle as O

    ref = Path(O.REF_SRC)
    gxx = shutil.which("g++")
    if gxx is None or not (ref / "factorize_electrical_system.h").exists():
        pytest.skip("needs g++ and the reference sources")
    text = (ROOT / "INTEGRATION.md").read_text()
    block = re.search(r"```cpp\n(.*?)```", text[text.index("## Shim"):], re.S)
    assert block, "no shim block"
    src = tmp_path / "pvglu_shim.cpp"
    src.write_text(block.group(1))
    cuda_inc = Path(shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc").resolve().parent.parent
    subprocess.run([gxx, "-std=c++17", "-fsyntax-only", "-Wall", "-I", str(ref), "-I",
                    str(ROOT / "include"), "-I", str(cuda_inc / "include"), str(src)],
                   check=True, timeout=120)
