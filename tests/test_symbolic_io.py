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


def _fnv1a(data: bytes) -> int:
    """64-bit FNV-1a (the dump's checksum)."""
    h = 0xCBF29CE484222325
    for c in data:
        h ^= c
        h = (h * 0x100000001B3) & 0xFFFFFFFFFFFFFFFF
    return h


def _array_offsets(raw: bytes) -> dict[str, tuple[int, int, int]]:
    """name -> (byte offset of the elements, element size, count) of a dump."""
    import struct

    pos = 8 + 4 + 4 + 7 * 8 + 8
    (count,) = struct.unpack_from("<I", raw, pos)
    pos += 4
    out = {}
    for _ in range(count):
        (ln,) = struct.unpack_from("<H", raw, pos)
        pos += 2
        name = raw[pos:pos + ln].decode()
        pos += ln
        es = raw[pos]
        pos += 1
        (cnt,) = struct.unpack_from("<Q", raw, pos)
        pos += 8
        out[name] = (pos, es, cnt)
        pos += es * cnt
    assert pos == len(raw) - 8
    return out


def test_damaged_files_fuzz(tmp_path):
    """Random single-byte flips and truncations are all refused."""
    p = Plant(1, 2, 5)
    s = Symbolic(p.rowptr, p.colidx)
    path = tmp_path / "s.pvs"
    s.save(path)
    raw = path.read_bytes()
    rng = np.random.default_rng(7)
    for k in range(150):
        bad = bytearray(raw)
        if k % 3 == 2:
            bad = bad[: int(rng.integers(0, len(raw)))]
        else:
            bad[int(rng.integers(0, len(raw)))] ^= 1 << int(rng.integers(0, 8))
        f = tmp_path / f"bad{k}.pvs"
        f.write_bytes(bytes(bad))
        with pytest.raises(PvgluError):
            Symbolic.load(f)


def test_out_of_range_content_with_valid_checksum_is_refused(tmp_path):
    """A dump whose checksum matches but whose index arrays point outside the
    analysis (a value past n or nnz, or negative) is refused by the range
    checks behind the checksum."""
    import struct

    p = Plant(1, 2, 5)
    s = Symbolic(p.rowptr, p.colidx)
    path = tmp_path / "s.pvs"
    s.save(path)
    raw = path.read_bytes()
    arrays = _array_offsets(raw)
    checked = 0
    for name, (off, es, cnt) in arrays.items():
        if es != 4 or cnt == 0:
            continue
        for value in (10 ** 9, -7):
            bad = bytearray(raw)
            struct.pack_into("<i", bad, off + 4 * (cnt // 2), value)
            struct.pack_into("<Q", bad, len(bad) - 8, _fnv1a(bytes(bad[:-8])))
            f = tmp_path / f"{name}_{value}.pvs"
            f.write_bytes(bytes(bad))
            with pytest.raises(PvgluError):
                Symbolic.load(f)
            checked += 1
    assert checked >= 20


def test_counts_beyond_int_with_valid_checksum_are_refused(tmp_path):
    """The dump stores n, the row-swap count and the involution flag as
    int64; values that an int cannot hold (n = 2^32 + n would truncate to n
    and pass every array check) are refused, not narrowed."""
    import struct

    p = Plant(1, 2, 5)
    s = Symbolic(p.rowptr, p.colidx)
    path = tmp_path / "s.pvs"
    s.save(path)
    raw = path.read_bytes()
    head = 8 + 4 + 4  # magic, version, byte order; then n, nnz_a, nnz_lu, row_swaps, invol
    (n,) = struct.unpack_from("<q", raw, head)
    for slot, value in ((0, (1 << 32) + n), (0, -1), (3, (1 << 32)), (4, 2), (4, -1)):
        bad = bytearray(raw)
        struct.pack_into("<q", bad, head + 8 * slot, value)
        struct.pack_into("<Q", bad, len(bad) - 8, _fnv1a(bytes(bad[:-8])))
        f = tmp_path / f"count{slot}_{value}.pvs"
        f.write_bytes(bytes(bad))
        with pytest.raises(PvgluError):
            Symbolic.load(f)
