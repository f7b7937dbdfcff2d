"""Symbolic analysis parity (CPU): product and oracle against the reference.

Golden fixtures hold the reference's own outputs (tests/golden/make_golden.py
runs the reference code); every symbolic array must match bit for bit.
"""
from __future__ import annotations

import numpy as np
import pytest
from conftest import golden_names, load_golden, rel_err

import matrices as M
from oracle import oracle as O
from phdthesis_albertojimenezruiz_gb300 import Plant, PvgluError, Symbolic

REF_ARRAYS = O.ARRAYS


@pytest.mark.parametrize("name", golden_names())
def test_product_symbolic_matches_reference(name):
    g = load_golden(name)
    s = Symbolic(g["rowptr"], g["colidx"], g["perm_amd"])
    got = s.arrays()
    for k in REF_ARRAYS:
        assert np.array_equal(got[k], g[k]), f"{name}: {k} differs"
    # Derived orderings follow from P and Q.
    assert np.array_equal(got["row_orig"], g["perm_amd"][g["perm_rows"]])
    assert np.array_equal(got["col_orig"], g["perm_amd"])


@pytest.mark.parametrize("name", golden_names())
def test_oracle_port_pinned_to_reference(name):
    """The CPU restatement reproduces the reference bit for bit: symbolic arrays,
    scattered values, both GLU orders and the solve."""
    g = load_golden(name)
    o = O.Port(g["rowptr"], g["colidx"], g["perm_amd"])
    got = o.arrays()
    for k in REF_ARRAYS:
        assert np.array_equal(got[k], g[k]), f"{name}: {k} differs"
    csc = o.scatter(g["a"])
    assert np.array_equal(csc, g["csc_in"])
    assert np.array_equal(o.refactor(csc, sequential=True), g["lu_seq"])
    assert np.array_equal(o.refactor(csc, sequential=False), g["lu_levels"])
    lu = g["lu_seq"]
    n = len(g["rowptr"]) - 1
    t = np.empty(n)
    t[np.argsort(g["perm_amd"])] = g["b"]
    w = np.empty(n)
    w[g["perm_rows"]] = t
    assert np.array_equal(o.solve(lu, w), g["x_perm"])


@pytest.mark.parametrize("name", golden_names())
def test_hazard_count_predicts_level_order_validity(name):
    """Where the reference's right-looking level schedule has no hazard, its
    level-ordered factors equal the sequential ones; where it has hazards
    (unsymmetric patterns) they do not, and the sequential factors are the
    valid LU (the kernels here compute the sequential result)."""
    g = load_golden(name)
    s = Symbolic(g["rowptr"], g["colidx"], g["perm_amd"])
    err = rel_err(g["lu_levels"], g["lu_seq"])
    if s.info["right_looking_hazards"] == 0:
        assert err <= 1e-12
    # A hazard is a pair that the parallel schedule may run out of order; the
    # reference's CPU walk of a level is serial, so only some hazards change
    # its result.  The unsymmetric random pattern is one where they do.
    if name.startswith("random"):
        assert s.info["right_looking_hazards"] > 0 and err > 1e-6


@pytest.mark.parametrize("dims", [(4, 8, 20), (10, 16, 20), (50, 24, 28)])
def test_product_vs_port_own_ordering(dims):
    """With the built-in ordering (no AMD), the oracle fed the same P agrees
    with every product array: the symbolic pipeline after the ordering is
    independent of where P came from."""
    p = Plant(*dims)
    s = Symbolic(p.rowptr, p.colidx)
    o = O.Port(p.rowptr, p.colidx, s.array("perm_amd"))
    got, want = s.arrays(), o.arrays()
    for k in REF_ARRAYS:
        assert np.array_equal(got[k], want[k]), k
    assert s.info["right_looking_hazards"] == 0


@pytest.mark.parametrize("fixture,tag,make", [
    ("plant_amd.npz", "50x24x28", lambda: (lambda p: (p.rowptr, p.colidx))(Plant(50, 24, 28))),
    ("block_plant_amd.npz", "7x50x50", lambda: M.block((7, 50, 50))[:2]),
])
def test_reference_ordering_reproduces_reference_counts(fixture, tag, make):
    """With the reference's own AMD ordering (fixtures made by the reference's
    code), the analysis gives the reference's fill and level counts, and the
    oracle's restatement the same arrays."""
    from conftest import GOLDEN

    with np.load(GOLDEN / "orderings" / fixture) as z:
        perm = z[f"perm_{tag}"]
        want = {k: int(z[f"{k}_{tag}"]) for k in ("nnz_lu", "lu_levels", "u_levels")}
    rp, ci = make()
    s = Symbolic(rp, ci, perm)
    assert int(s.nnz_lu) == want["nnz_lu"]
    assert s.info["lu_levels"] == want["lu_levels"] and s.info["u_levels"] == want["u_levels"]
    assert np.array_equal(s.array("perm_amd"), perm)
    if fixture == "plant_amd.npz":
        got, ref = s.arrays(), O.Port(rp, ci, perm).arrays()
        for k in REF_ARRAYS:
            assert np.array_equal(got[k], ref[k]), k


@pytest.mark.parametrize("case", ["mesh_30x30", "random_1500"])
def test_product_vs_port_fill_heavy(case):
    rp, ci, _, _ = M.CASES[case]()
    s = Symbolic(rp, ci)
    o = O.Port(rp, ci, s.array("perm_amd"))
    got, want = s.arrays(), o.arrays()
    for k in REF_ARRAYS:
        assert np.array_equal(got[k], want[k]), k


def test_transposed_levels_are_valid_schedule():
    rp, ci, _, _ = M.CASES["random_1500"]()
    s = Symbolic(rp, ci)
    a = s.arrays()
    o = O.Port(rp, ci, a["perm_amd"])
    assert np.array_equal(a["lt_sl"], o.get("lt_sl"))
    assert np.array_equal(a["lt_cols"], o.get("lt_cols"))
    # every L^T dependency of j (rows i > j with L(i,j)) is scheduled first
    n = s.n
    level = np.empty(n, np.int64)
    chain = np.empty(n, np.int64)
    pos = np.empty(n, np.int64)
    for lv in range(len(a["lt_sl"]) - 1):
        for c in range(a["lt_sl"][lv], a["lt_sl"][lv + 1]):
            for t in range(a["lt_sc"][c], a["lt_sc"][c + 1]):
                j = a["lt_cols"][t]
                level[j], chain[j], pos[j] = lv, c, t
    cp, rows = a["csc_colptr"], a["csc_row"]
    for j in range(n):
        for q in range(cp[j], cp[j + 1]):
            i = rows[q]
            if i > j:
                assert level[i] < level[j] or (chain[i] == chain[j] and pos[i] < pos[j])


def test_update_targets_cover_flop_count():
    rp, ci, _, _ = M.CASES["mesh_20x20"]()
    s = Symbolic(rp, ci)
    a = s.arrays()
    cp, dg = a["csc_colptr"], a["diag_slot"]
    rpl = a["csr_rowptr"]
    ds = a["csr_diag_start"]
    nl = cp[1:] - (dg + 1)
    nu = rpl[1:] - ds
    assert s.info["update_count"] == int(np.sum(nl * nu))


def test_bad_inputs_raise():
    rp = np.array([0, 1, 2], np.int32)
    with pytest.raises(PvgluError) as e:
        Symbolic(rp, np.array([0, 0], np.int32), [0, 0])
    assert e.value.code == 1  # not a permutation
    with pytest.raises(PvgluError) as e:
        Symbolic(np.array([0, 2, 3], np.int32), np.array([0, 0, 1], np.int32))
    assert e.value.code == 1  # duplicate entry
    with pytest.raises(PvgluError) as e:
        Symbolic(np.array([0, 1, 2], np.int32), np.array([0, 5], np.int32))
    assert e.value.code == 1  # column out of range
    # structurally singular: column 1 is empty, so row 1 can neither be filled
    # at its diagonal nor exchanged with a later row (004b:82)
    with pytest.raises(PvgluError) as e:
        Symbolic(np.array([0, 1, 2], np.int32), np.array([0, 0], np.int32), [0, 1])
    assert e.value.code == 2


def test_single_unknown_and_diagonal_matrix():
    s = Symbolic(np.array([0, 1], np.int32), np.array([0], np.int32))
    assert s.n == 1 and s.nnz_lu == 1
    n = 50
    s = Symbolic(np.arange(n + 1, dtype=np.int32), np.arange(n, dtype=np.int32))
    assert s.info["lu_levels"] == 1 and s.info["lu_chains"] == n


def test_product_vs_port_random_patterns():
    """Fuzz: 288 random unsymmetric MNA patterns (sizes 6-150, node degrees 2-5,
    0-6 voltage sources, so zero diagonals and row exchanges) analysed with the
    built-in ordering and with a random caller ordering; every array equals
    the oracle's restatement fed the same P."""
    import itertools

    rng = np.random.default_rng(123)
    for n, deg, src, seed in itertools.product([6, 12, 40, 150], [2.0, 3.0, 5.0], [0, 1, 3, 6],
                                               range(6)):
        rp, ci, _, _ = M.random_mna(n, deg, src, seed)
        for perm in (None, rng.permutation(len(rp) - 1).astype(np.int32)):
            s = Symbolic(rp, ci, perm)
            o = O.Port(rp, ci, s.array("perm_amd"))
            got, want = s.arrays(), o.arrays()
            for k in REF_ARRAYS:
                assert np.array_equal(got[k], want[k]), (n, deg, src, seed, perm is None, k)


def test_malformed_patterns_are_refused_not_crashed():
    """Fuzz of the analysis entry point with malformed CSR (out-of-range and
    duplicate columns, non-monotone row pointers, missing diagonals, bad
    permutations) and with valid random patterns: every call returns an
    analysis or raises PvgluError; accepted analyses have a permutation
    ordering and schedule every column once."""
    from phdthesis_albertojimenezruiz_gb300 import PvgluError

    rng = np.random.default_rng(11)
    accepted = refused = 0
    for it in range(1200):
        n = int(rng.integers(0, 12))
        kind = it % 5
        perm = None
        if kind == 0:
            counts = rng.integers(0, 5, n)
            rp = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
            ci = rng.integers(-2, n + 2, int(rp[-1])).astype(np.int32)
        elif kind == 1:
            rp = rng.integers(-3, 10, n + 1).astype(np.int32)
            ci = np.zeros(32, dtype=np.int32)
        else:
            rows = []
            for i in range(n):
                extra = rng.integers(0, n, int(rng.integers(0, 4))).tolist() if n else []
                rows.append(sorted(set(([i] if kind != 3 else []) + extra)))
            rp = np.concatenate([[0], np.cumsum([len(r) for r in rows])]).astype(np.int32)
            ci = np.array([c for r in rows for c in r] + [0], dtype=np.int32)
            if kind == 4 and n:
                perm = rng.integers(-1, n + 1, n).astype(np.int32)
        try:
            s = Symbolic(rp, ci, perm)
        except PvgluError:
            refused += 1
            continue
        accepted += 1
        assert np.array_equal(np.sort(s.array("perm_amd")), np.arange(s.n))
        assert np.array_equal(np.sort(s.array("lu_cols")), np.arange(s.n))
    assert accepted > 100 and refused > 100
