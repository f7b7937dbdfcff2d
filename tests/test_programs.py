"""Chain-program compiler (CPU): for every program kind and several table
budgets, the programs of plants and of the golden matrices satisfy the
invariants the device executors rely on -- every load, carry and operation
operand inside its segment's table, each table within its level's budget,
own rows first, read-only values never written back (program_invariants.cpp,
compiled here against the host sources)."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest
from conftest import golden_names, load_golden

from phdthesis_albertojimenezruiz_gb300 import Plant

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "phdthesis_albertojimenezruiz_gb300" / "csrc"


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path_factory.mktemp("prog") / "program_invariants"
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", str(CSRC),
                    str(Path(__file__).with_name("program_invariants.cpp")),
                    str(CSRC / "symbolic.cpp"), str(CSRC / "programs.cpp"), "-o", str(exe)],
                   check=True, timeout=300)
    return exe


def run(checker, tmp_path, rowptr, colidx):
    rp, ci = tmp_path / "rowptr.bin", tmp_path / "colidx.bin"
    np.asarray(rowptr, dtype=np.int32).tofile(rp)
    np.asarray(colidx, dtype=np.int32).tofile(ci)
    out = subprocess.run([str(checker), str(len(rowptr) - 1), str(rp), str(ci)],
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr


@pytest.mark.parametrize("dims", [(1, 1, 3), (1, 2, 2), (4, 8, 20), (10, 16, 20), (50, 24, 28)])
def test_plant_programs(checker, tmp_path, dims):
    p = Plant(*dims)
    run(checker, tmp_path, p.rowptr, p.colidx)


@pytest.mark.parametrize("name", golden_names())
def test_golden_programs(checker, tmp_path, name):
    g = load_golden(name)
    run(checker, tmp_path, g["rowptr"], g["colidx"])


@pytest.mark.parametrize("n,deg,src,seed", [(40, 3.0, 3, 1), (150, 5.0, 6, 2), (300, 2.0, 0, 3)])
def test_random_pattern_programs(checker, tmp_path, n, deg, src, seed):
    import matrices as M

    rp, ci, _, _ = M.random_mna(n, deg, src, seed)
    run(checker, tmp_path, rp, ci)
