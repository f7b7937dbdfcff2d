"""Symbolic dump format (pvglu_symbolic_save / pvglu_symbolic_load): round
trips keep every array and the info bit for bit; damaged files are refused."""
from __future__ import annotations

import numpy as np
import pytest
from conftest import golden_names, load_golden

from phdthesis_albertojimenezruiz_gb300 import Plant, PvgluError, Symbolic


def _same(s: Symbolic, t: Symbolic) -> None:
    a, b = s.arrays(), t.arrays()
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    assert s.info == t.info


@pytest.mark.parametrize("dims", [(1, 2, 2), (4, 8, 20), (50, 24, 28)])
def test_plant_round_trip(tmp_path, dims):
    p = Plant(*dims)
    s = Symbolic(p.rowptr, p.colidx)
    s.save(tmp_path / "s.pvs")
    _same(s, Symbolic.load(tmp_path / "s.pvs"))


@pytest.mark.parametrize("name", golden_names())
def test_golden_round_trip(tmp_path, name):
    g = load_golden(name)
    s = Symbolic(g["rowptr"], g["colidx"], g["perm_amd"])
    s.save(tmp_path / "g.pvs")
    t = Symbolic.load(tmp_path / "g.pvs")
    _same(s, t)
    assert np.array_equal(t.array("perm_rows"), g["perm_rows"])


def test_damaged_files_are_refused(tmp_path):
    p = Plant(2, 4, 10)
    s = Symbolic(p.rowptr, p.colidx)
    path = tmp_path / "s.pvs"
    s.save(path)
    raw = bytearray(path.read_bytes())
    flipped = bytearray(raw)
    flipped[len(raw) // 2] ^= 0x40
    (tmp_path / "flip.pvs").write_bytes(bytes(flipped))
    (tmp_path / "short.pvs").write_bytes(bytes(raw[: len(raw) - 100]))
    (tmp_path / "magic.pvs").write_bytes(b"NOTADUMP" + bytes(raw[8:]))
    (tmp_path / "empty.pvs").write_bytes(b"")
    for bad in ("flip.pvs", "short.pvs", "magic.pvs", "empty.pvs", "missing.pvs"):
        with pytest.raises(PvgluError):
            Symbolic.load(tmp_path / bad)
