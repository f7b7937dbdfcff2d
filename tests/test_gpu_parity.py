"""GPU parity: the sm_103a scatter / refactor / solve kernels against the
reference's outputs (golden fixtures) and the CPU oracle, through the C ABI.

Tolerances: FP64 factors 1e-12 componentwise relative (floor 1e-6 x max|ref|,
conftest.rel_err); FP64 solutions 1e-12 normwise relative (conftest.norm_err:
entries that come out of a cancellation carry the rounding of the larger
terms); FP32 factors + FP64 refinement 1e-10 normwise relative against the
FP64 oracle solution.  The kernels fuse multiply-adds where the reference's
CPU code rounds twice, so bit equality is not expected for values.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest
from conftest import golden_names, load_golden, norm_err, rel_err

import matrices as M
from oracle import oracle as O
from phdthesis_albertojimenezruiz_gb300 import (FP32, FP64, SCHED_LEVELS, SCHED_PERSISTENT,
                                                SCHED_THREAD_CHAIN, Numeric, Plant, Symbolic)
from phdthesis_albertojimenezruiz_gb300 import _native as N

pytestmark = pytest.mark.gpu
SCHEDULES = [SCHED_LEVELS, SCHED_PERSISTENT, SCHED_THREAD_CHAIN]
TOL64 = 1e-12


class _DevView:
    """A CUDA array interface over library-owned device memory."""

    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"shape": shape, "typestr": typestr,
                                         "data": (ptr, False), "version": 3}


def values_of(num: Numeric, count: int) -> np.ndarray:
    import torch

    ts = "<f8" if num.precision == FP64 else "<f4"
    t = torch.as_tensor(_DevView(num.values_ptr(), (count * num.ld,), ts), device="cuda")
    torch.cuda.synchronize()
    return t.cpu().numpy().astype(np.float64).reshape(count, num.ld)


def dev(a, dtype=None):
    import torch

    t = torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).cuda()
    return t


def pad_cols(a: np.ndarray, ld: int) -> np.ndarray:
    """[rows, S] -> [rows, ld] (padding columns zero)."""
    out = np.zeros((a.shape[0], ld))
    out[:, : a.shape[1]] = a
    return out


def to_perm(g, b):
    n = len(b)
    t = np.empty(n)
    t[np.argsort(g["perm_amd"])] = b
    w = np.empty(n)
    w[g["perm_rows"]] = t
    return w


@pytest.mark.parametrize("schedule", SCHEDULES)
@pytest.mark.parametrize("name", golden_names())
def test_golden_single_fp64(cuda, name, schedule):
    import torch

    g = load_golden(name)
    s = Symbolic(g["rowptr"], g["colidx"], g["perm_amd"])
    num = Numeric(s, 1, FP64, schedule)
    nnz = int(s.nnz_lu)
    num.scatter(dev(g["a"]))
    assert np.array_equal(values_of(num, nnz)[:, 0], g["csc_in"])  # (a) exact copy
    num.refactor()
    assert num.check() == (0, -1, -1)
    lu = values_of(num, nnz)[:, 0]
    assert rel_err(lu, g["lu_seq"]) <= TOL64
    # (c) permuted-space solve: triangular_substitution_LU_CUDA semantics
    x = dev(to_perm(g, g["b"]))
    num.solve(x)
    assert norm_err(x.cpu().numpy(), g["x_perm"]) <= TOL64
    # original-order solve
    x = dev(g["b"])
    num.solve(x, original=True)
    torch.cuda.synchronize()
    assert norm_err(x.cpu().numpy(), g["x"]) <= TOL64


@pytest.mark.parametrize("schedule", SCHEDULES)
@pytest.mark.parametrize("name", golden_names())
def test_golden_fp64_bit_exact(cuda, name, schedule):
    """Stronger than the 1e-12 bar: the FP64 kernels apply every update to an
    entry in the reference's sequential order with separately rounded
    multiply and subtract, so factors and solution equal the reference's
    GLU_CSC_CPU_sequential + Substitute_LU_Vector_b_CSC_CPU bit for bit."""
    g = load_golden(name)
    s = Symbolic(g["rowptr"], g["colidx"], g["perm_amd"])
    num = Numeric(s, 1, FP64, schedule)
    num.scatter(dev(g["a"]))
    x = dev(to_perm(g, g["b"]))
    num.refactor_solve(x)
    assert np.array_equal(values_of(num, int(s.nnz_lu))[:, 0], g["lu_seq"])
    assert np.array_equal(x.cpu().numpy(), g["x_perm"])


@pytest.mark.parametrize("schedule", SCHEDULES)
@pytest.mark.parametrize("name", golden_names())
def test_transposed_solve_fp64(cuda, name, schedule):
    g = load_golden(name)
    s = Symbolic(g["rowptr"], g["colidx"], g["perm_amd"])
    o = O.Port(g["rowptr"], g["colidx"], g["perm_amd"])
    num = Numeric(s, 1, FP64, schedule)
    num.scatter(dev(g["a"]))
    num.refactor()
    rng = np.random.default_rng(7)
    b = rng.uniform(-1, 1, s.n)
    x = dev(b)
    num.solve(x, transpose=True)
    want = o.solve_transposed(g["lu_seq"], b)
    assert norm_err(x.cpu().numpy(), want) <= TOL64
    # original order: J^T lam = b
    import scipy.sparse as sp

    J = sp.csr_matrix((g["a"], g["colidx"], g["rowptr"]), shape=(s.n, s.n))
    lam = dev(b)
    num.solve(lam, transpose=True, original=True)
    lam = lam.cpu().numpy()
    assert np.abs(J.T @ lam - b).max() <= 1e-10 * (np.abs(J).max() * np.abs(lam).max() + 1)


@pytest.mark.parametrize("schedule", SCHEDULES)
@pytest.mark.parametrize("case", ["mesh_30x30", "random_1500"])
def test_fill_heavy_vs_oracle(cuda, case, schedule):
    rp, ci, a, b = M.CASES[case]()
    s = Symbolic(rp, ci)
    o = O.Port(rp, ci, s.array("perm_amd"))
    num = Numeric(s, 1, FP64, schedule)
    num.scatter(dev(a))
    num.refactor()
    lu_ref = o.refactor(o.scatter(a), sequential=True)
    assert rel_err(values_of(num, int(s.nnz_lu))[:, 0], lu_ref) <= TOL64
    x = dev(b)
    num.solve(x, original=True)
    _, x_ref = o.scatter_refactor_solve(a, b)
    assert norm_err(x.cpu().numpy(), x_ref) <= TOL64


@pytest.mark.parametrize("schedule", SCHEDULES)
@pytest.mark.parametrize("dims,S", [((10, 16, 20), 37), ((4, 8, 20), 64)])
def test_batched_plant_fp64(cuda, dims, S, schedule):
    p = Plant(*dims)
    s = Symbolic(p.rowptr, p.colidx)
    o = O.Port(p.rowptr, p.colidx, s.array("perm_amd"))
    num = Numeric(s, S, FP64, schedule)
    a, b = M.plant_batch(p, S, seed0=11, preset="c3")
    num.scatter(dev(pad_cols(a, num.ld)))
    num.refactor()
    assert num.check()[0] == 0
    lu = values_of(num, int(s.nnz_lu))
    x = dev(pad_cols(b, num.ld))
    num.solve(x, original=True)
    x = x.cpu().numpy().reshape(s.n, num.ld)
    for k in range(S):
        lu_ref, x_ref = o.scatter_refactor_solve(a[:, k], b[:, k])
        assert rel_err(lu[:, k], lu_ref) <= TOL64, k
        assert norm_err(x[:, k], x_ref) <= TOL64, k


@pytest.mark.parametrize("ld_scenarios", [1, 40])
def test_fp32_scatter_rounds_like_numpy(cuda, ld_scenarios):
    """The FP32 scatter converts FP64 values on the integer pipes: round to
    nearest even for normal floats, signed zero below 2^-126, +-inf past the
    float range; numpy's float32 cast is the reference for everything else."""
    p = Plant(2, 4, 10)
    s = Symbolic(p.rowptr, p.colidx)
    num = Numeric(s, ld_scenarios, FP32, SCHED_LEVELS)
    rng = np.random.default_rng(4)
    a = rng.standard_normal((int(s.nnz_a), ld_scenarios)) * 10.0 ** rng.integers(-45, 45, (
        int(s.nnz_a), ld_scenarios))
    a[:8, 0] = [0.0, -0.0, 1.0 + 2.0 ** -24, 1.0 + 3 * 2.0 ** -24, 3.5e38, -1e39, 1e-40, np.nan]
    num.scatter(dev(pad_cols(a, num.ld)))
    got = values_of(num, int(s.nnz_lu))[:, :ld_scenarios]
    src = s.array("slot_src")
    want = np.zeros_like(got)
    with np.errstate(over="ignore"):
        cast = a.astype(np.float32).astype(np.float64)
    cast[np.abs(a) < 2.0 ** -126] = 0.0
    want[src >= 0] = cast[src[src >= 0]]
    same = (got == want) | (np.isnan(got) & np.isnan(want))
    assert same.all(), np.argwhere(~same)[:5]


@pytest.mark.parametrize("schedule", SCHEDULES)
def test_plant_35k_fp64(cuda, schedule):
    """The ~35k-unknown plant (50 x 24 x 28): single instance and a batch."""
    p = Plant(50, 24, 28)
    s = Symbolic(p.rowptr, p.colidx)
    o = O.Port(p.rowptr, p.colidx, s.array("perm_amd"))
    S = 8
    a, b = M.plant_batch(p, S, seed0=100, preset="c2")
    for count in (1, S):
        num = Numeric(s, count, FP64, schedule)
        num.scatter(dev(pad_cols(a[:, :count], num.ld)))
        num.refactor()
        x = dev(pad_cols(b[:, :count], num.ld))
        num.solve(x, original=True)
        x = x.cpu().numpy().reshape(s.n, num.ld)
        lu = values_of(num, int(s.nnz_lu))
        for k in range(count):
            lu_ref, x_ref = o.scatter_refactor_solve(a[:, k], b[:, k])
            assert rel_err(lu[:, k], lu_ref) <= TOL64
            assert norm_err(x[:, k], x_ref) <= TOL64


@pytest.mark.parametrize("schedule", SCHEDULES)
def test_fp32_refinement_35k(cuda, schedule):
    import torch

    p = Plant(50, 24, 28)
    s = Symbolic(p.rowptr, p.colidx)
    o = O.Port(p.rowptr, p.colidx, s.array("perm_amd"))
    S = 40
    a, b = M.plant_batch(p, S, seed0=300, preset="c3")
    num = Numeric(s, S, FP32, schedule)
    a_dev = dev(pad_cols(a, num.ld))
    b_dev = dev(pad_cols(b, num.ld))
    num.scatter(a_dev)
    num.refactor()
    x = torch.zeros_like(b_dev)
    sweeps = torch.zeros(num.ld, dtype=torch.int32, device="cuda")
    # tol sits above the FP64 rounding floor of the residual (about cond x eps64
    # relative for this plant); below it the corrections stop shrinking.
    num.solve_refined(a_dev, b_dev, x, tol=1e-12, max_sweeps=10, sweeps=sweeps)
    torch.cuda.synchronize()
    x = x.cpu().numpy()
    sw = sweeps.cpu().numpy()[:S]
    assert (sw > 0).all(), sw
    for k in range(S):
        _, x_ref = o.scatter_refactor_solve(a[:, k], b[:, k])
        err = np.abs(x[:, k] - x_ref).max() / np.abs(x_ref).max()
        assert err <= 1e-10, (k, err, sw[k])


@pytest.mark.parametrize("schedule", SCHEDULES)
@pytest.mark.parametrize("dims,preset", [((120, 24, 28), "c3"), ((200, 24, 28), "c4")])
def test_large_plants_fp64_vs_oracle(cuda, dims, preset, schedule):
    """The 84k-unknown plant of the three-size batch (120 x 24 x 28) and the
    135k-unknown plant of the precision configuration (200 x 24 x 28), FP64,
    single instance and a batch of 3, against the oracle scenario by
    scenario: factors 1e-12 componentwise, solutions 1e-12 normwise."""
    p = Plant(*dims)
    s = Symbolic(p.rowptr, p.colidx)
    o = O.Port(p.rowptr, p.colidx, s.array("perm_amd"))
    S = 3
    a, b = M.plant_batch(p, S, seed0=4100 + dims[0], preset=preset)
    refs = [o.scatter_refactor_solve(a[:, k], b[:, k]) for k in range(S)]
    for count in (1, S):
        num = Numeric(s, count, FP64, schedule)
        num.scatter(dev(pad_cols(a[:, :count], num.ld)))
        num.refactor()
        assert num.check()[0] == 0
        x = dev(pad_cols(b[:, :count], num.ld))
        num.solve(x, original=True)
        x = x.cpu().numpy().reshape(s.n, num.ld)
        lu = values_of(num, int(s.nnz_lu))
        for k in range(count):
            assert rel_err(lu[:, k], refs[k][0]) <= TOL64, (count, k)
            assert norm_err(x[:, k], refs[k][1]) <= TOL64, (count, k)


@pytest.mark.parametrize("schedule", [SCHED_LEVELS, SCHED_PERSISTENT])
@pytest.mark.parametrize("dims,preset", [((120, 24, 28), "c3"), ((200, 24, 28), "c4")])
def test_large_plants_fp32_refinement_vs_oracle(cuda, dims, preset, schedule):
    """FP32 factors + FP64 refinement on the 84k and 135k plants: every
    scenario within 1e-10 of the oracle's FP64 solution (normwise)."""
    import torch

    p = Plant(*dims)
    s = Symbolic(p.rowptr, p.colidx)
    o = O.Port(p.rowptr, p.colidx, s.array("perm_amd"))
    S = 4
    a, b = M.plant_batch(p, S, seed0=4300 + dims[0], preset=preset)
    num = Numeric(s, S, FP32, schedule)
    a_dev = dev(pad_cols(a, num.ld))
    b_dev = dev(pad_cols(b, num.ld))
    num.scatter(a_dev)
    num.refactor()
    assert num.check()[0] == 0
    x = torch.zeros_like(b_dev)
    sweeps = torch.zeros(num.ld, dtype=torch.int32, device="cuda")
    num.solve_refined(a_dev, b_dev, x, tol=1e-12, max_sweeps=10, sweeps=sweeps)
    torch.cuda.synchronize()
    x = x.cpu().numpy()
    sw = sweeps.cpu().numpy()[:S]
    assert (sw > 0).all(), sw
    for k in range(S):
        _, x_ref = o.scatter_refactor_solve(a[:, k], b[:, k])
        assert norm_err(x[:, k], x_ref) <= 1e-10, (k, sw[k])


def block_batch(dims, S: int, seed0: int):
    """A values [nnz_a, S] and b [n, S] of the reference-topology plant, one
    seed (diode operating point) per scenario, same pattern."""
    from phdthesis_albertojimenezruiz_gb300.plant import block_plant

    cols = [block_plant(*dims, seed=seed0 + k) for k in range(S)]
    return np.stack([c[2] for c in cols], 1), np.stack([c[3] for c in cols], 1)


def block_ordering(tag: str):
    """The reference's AMD ordering of the reference-topology plant (fixture)."""
    from conftest import GOLDEN

    with np.load(GOLDEN / "orderings" / "block_plant_amd.npz") as z:
        return z[f"perm_{tag}"], int(z[f"nnz_lu_{tag}"]), int(z[f"u_levels_{tag}"])


@pytest.mark.parametrize("schedule", [SCHED_LEVELS, SCHED_PERSISTENT])
@pytest.mark.parametrize("S,max_locals", [(1, 8), (1, 40), (1, 0), (64, 8), (130, 16)])
@pytest.mark.parametrize("name", ["block_1x20x20", "mesh_20x20", "random_300"])
def test_wide_units_bit_exact(cuda, name, S, max_locals, schedule):
    """Columns and rows too wide for the table run as WIDE program levels
    (a block per unit: chain-scheduled gather for the refactorization,
    ordered block sums for the solves).  Small tables make many units wide;
    FP64 factors and solutions stay bit-identical to the reference's
    sequential GLU and substitution for every scenario, and the transposed
    solve matches the oracle."""
    import torch

    g = load_golden(name)
    s = Symbolic(g["rowptr"], g["colidx"], g["perm_amd"])
    o = O.Port(g["rowptr"], g["colidx"], g["perm_amd"])
    num = Numeric(s, S, FP64, schedule, max_locals=max_locals)
    a = np.repeat(g["a"][:, None], S, axis=1)
    num.scatter(dev(pad_cols(a, num.ld)))
    num.refactor()
    assert num.check()[0] == 0
    lu = values_of(num, int(s.nnz_lu))[:, :S]
    assert np.array_equal(lu, np.repeat(g["lu_seq"][:, None], S, axis=1))
    b = np.repeat(to_perm(g, g["b"])[:, None], S, axis=1)
    x = dev(pad_cols(b, num.ld))
    num.solve(x)
    xs = x.cpu().numpy().reshape(s.n, num.ld)[:, :S]
    assert np.array_equal(xs, np.repeat(g["x_perm"][:, None], S, axis=1))
    rng = np.random.default_rng(9)
    bt = rng.uniform(-1, 1, s.n)
    xt = dev(pad_cols(np.repeat(bt[:, None], S, axis=1), num.ld))
    num.solve(xt, transpose=True)
    torch.cuda.synchronize()
    want = o.solve_transposed(g["lu_seq"], bt)
    got = xt.cpu().numpy().reshape(s.n, num.ld)
    for k in sorted({0, S - 1}):
        assert np.array_equal(got[:, k], want), k


@pytest.mark.parametrize("schedule", [SCHED_LEVELS, SCHED_PERSISTENT])
@pytest.mark.parametrize("S", [1, 64])
def test_reference_topology_plant_fp64(cuda, S, schedule):
    """The reference's own plant topology (1 x 50 x 50 panels, strings between
    shared bus nodes, internal diode nodes) with the reference's AMD ordering:
    the analysis reproduces the reference's fill and level counts, the bus
    columns and rows (2,500 entries) run as wide units, and FP64 factors and
    solutions equal the oracle's (the reference's sequential arithmetic) bit
    for bit."""
    from phdthesis_albertojimenezruiz_gb300.plant import block_plant

    perm, nnz_lu, u_levels = block_ordering("1x50x50")
    a, b = block_batch((1, 50, 50), S, seed0=210)
    rp, ci, _, _ = block_plant(1, 50, 50)
    s = Symbolic(rp, ci, perm)
    assert int(s.nnz_lu) == nnz_lu and s.info["u_levels"] == u_levels
    o = O.Port(rp, ci, perm)
    num = Numeric(s, S, FP64, schedule)
    num.scatter(dev(pad_cols(a, num.ld)))
    num.refactor()
    assert num.check()[0] == 0
    x = dev(pad_cols(b, num.ld))
    num.solve(x, original=True)
    x = x.cpu().numpy().reshape(s.n, num.ld)
    lu = values_of(num, int(s.nnz_lu))
    for k in sorted({0, S // 2, S - 1}):
        lu_ref, x_ref = o.scatter_refactor_solve(a[:, k], b[:, k])
        assert np.array_equal(lu[:, k], lu_ref), k
        assert np.array_equal(x[:, k], x_ref), k


@pytest.mark.parametrize("schedule", [SCHED_LEVELS, SCHED_PERSISTENT])
def test_reference_topology_plant_fp32_refinement(cuda, schedule):
    """FP32 factors (wide units included) + FP64 refinement on the
    reference-topology plant: within 1e-10 of the oracle's FP64 solution."""
    import torch

    from phdthesis_albertojimenezruiz_gb300.plant import block_plant

    perm, _, _ = block_ordering("1x50x50")
    rp, ci, _, _ = block_plant(1, 50, 50)
    s = Symbolic(rp, ci, perm)
    o = O.Port(rp, ci, perm)
    S = 64
    a, b = block_batch((1, 50, 50), S, seed0=230)
    num = Numeric(s, S, FP32, schedule)
    a_dev = dev(pad_cols(a, num.ld))
    b_dev = dev(pad_cols(b, num.ld))
    num.scatter(a_dev)
    num.refactor()
    assert num.check()[0] == 0
    x = torch.zeros_like(b_dev)
    sweeps = torch.zeros(num.ld, dtype=torch.int32, device="cuda")
    num.solve_refined(a_dev, b_dev, x, tol=1e-12, max_sweeps=30, sweeps=sweeps)
    torch.cuda.synchronize()
    sw = sweeps.cpu().numpy()[:S]
    assert (sw > 0).all(), sw
    x = x.cpu().numpy()
    for k in (0, 31, 63):
        _, x_ref = o.scatter_refactor_solve(a[:, k], b[:, k])
        assert norm_err(x[:, k], x_ref) <= 1e-10, (k, sw[k])


def test_group_with_wide_members(cuda):
    """A size-class group whose members have WIDE levels: each member's wide
    levels run as their own launches, the rest grouped; bit-identical to the
    members alone."""
    import torch

    from phdthesis_albertojimenezruiz_gb300.glu import Group

    names = ["block_1x20x20", "mesh_20x20", "plant_c1"]
    members, refs, xs = [], [], []
    for name in names:
        g = load_golden(name)
        s = Symbolic(g["rowptr"], g["colidx"], g["perm_amd"])
        S = 64
        a = np.repeat(g["a"][:, None], S, axis=1)
        b = np.repeat(g["b"][:, None], S, axis=1)
        alone = Numeric(s, S, FP64, SCHED_LEVELS, max_locals=8)
        alone.scatter(dev(pad_cols(a, alone.ld)))
        xa = dev(pad_cols(b, alone.ld))
        alone.refactor()
        alone.solve(xa, original=True)
        torch.cuda.synchronize()
        refs.append((values_of(alone, int(s.nnz_lu)), xa.cpu().numpy(), int(s.nnz_lu)))
        grouped = Numeric(s, S, FP64, SCHED_LEVELS, max_locals=8)
        grouped.scatter(dev(pad_cols(a, grouped.ld)))
        members.append(grouped)
        xs.append(dev(pad_cols(b, grouped.ld)))
    grp = Group(members)
    grp.refactor_solve(xs, original=True)
    torch.cuda.synchronize()
    for h, x, (lu_ref, x_ref, nnz) in zip(members, xs, refs):
        assert h.check()[0] == 0
        assert np.array_equal(values_of(h, nnz)[:, :64], lu_ref[:, :64])
        assert np.array_equal(x.cpu().numpy().reshape(-1, h.ld)[:, :64],
                              x_ref.reshape(-1, h.ld)[:, :64])


@pytest.mark.parametrize("schedule", [SCHED_LEVELS, SCHED_PERSISTENT])
@pytest.mark.parametrize("merge,wide", [(1, 0), (0, 0), (2, 0), (1, 12), (0, 12), (2, 12)])
@pytest.mark.parametrize("S", [1, 64])
@pytest.mark.parametrize("name", ["block_1x20x20", "mesh_20x20"])
def test_every_tuning_bit_exact(cuda, name, S, merge, wide, schedule):
    """Every execution choice of pvglu_tuning (execution levels merged per
    unit, with ladder merging, or the level set's own; wide units at half the
    table or only where needed; each schedule) gives the reference's
    sequential FP64 factors and solution bit for bit."""
    g = load_golden(name)
    s = Symbolic(g["rowptr"], g["colidx"], g["perm_amd"])
    t = {"max_locals": 24, "wide_threshold": wide, "merge_chains": merge, "schedule": schedule}
    num = Numeric(s, S, FP64, tuning=t)
    a = np.repeat(g["a"][:, None], S, axis=1)
    num.scatter(dev(pad_cols(a, num.ld)))
    x = dev(pad_cols(np.repeat(to_perm(g, g["b"])[:, None], S, axis=1), num.ld))
    num.refactor_solve(x)
    assert num.check()[0] == 0
    lu = values_of(num, int(s.nnz_lu))[:, :S]
    assert np.array_equal(lu, np.repeat(g["lu_seq"][:, None], S, axis=1))
    xs = x.cpu().numpy().reshape(s.n, num.ld)[:, :S]
    assert np.array_equal(xs, np.repeat(g["x_perm"][:, None], S, axis=1))


@pytest.mark.parametrize("name,ladder", [("block_1x20x20", True), ("plant_c1", False)])
def test_default_chain_merging(cuda, name, ladder):
    """pvglu_numeric_create merges chains with the ladder rule where that
    halves the execution levels (the reference's plant topology: a U-solve
    level per string rung otherwise) and keeps the level set's own chains
    elsewhere; either way the FP64 solution is the reference's, bit for bit."""
    g = load_golden(name)
    s = Symbolic(g["rowptr"], g["colidx"], g["perm_amd"])
    base = {"max_locals": 0, "wide_threshold": 0, "schedule": SCHED_LEVELS}
    levels = {m: Numeric(s, 1, FP64, tuning=dict(base, merge_chains=m)).info["program_levels"]
              for m in (0, 2)}
    num = Numeric(s, 1, FP64)
    assert num.info["program_levels"] == levels[2 if ladder else 0]
    if ladder:
        assert 2 * levels[2] <= levels[0]
    num.scatter(dev(pad_cols(g["a"][:, None], num.ld)))
    x = dev(pad_cols(to_perm(g, g["b"])[:, None], num.ld))
    num.refactor_solve(x)
    assert num.check()[0] == 0
    assert np.array_equal(x.cpu().numpy().reshape(s.n, num.ld)[:, 0], g["x_perm"])


@pytest.mark.parametrize("name,S,precision", [("block_1x20x20", 1, FP64),
                                              ("block_1x20x20", 130, FP64),
                                              ("plant_c1", 64, FP32)])
def test_autotune_ex_picks_a_working_tuning(cuda, name, S, precision):
    from phdthesis_albertojimenezruiz_gb300.glu import autotune_ex

    g = load_golden(name)
    s = Symbolic(g["rowptr"], g["colidx"], g["perm_amd"])
    t, ms = autotune_ex(s, S, precision)
    assert ms > 0 and t["schedule"] in (SCHED_LEVELS, SCHED_PERSISTENT)
    assert t["merge_chains"] in (0, 1, 2) and t["wide_threshold"] >= 0
    num = Numeric(s, S, precision, tuning=t)
    a = np.repeat(g["a"][:, None], S, axis=1)
    num.scatter(dev(pad_cols(a, num.ld)))
    x = dev(pad_cols(np.repeat(to_perm(g, g["b"])[:, None], S, axis=1), num.ld),
            np.float64 if precision == FP64 else np.float32)
    num.refactor_solve(x)
    assert num.check()[0] == 0
    x = x.cpu().numpy().reshape(s.n, num.ld).astype(np.float64)
    want = g["x_perm"]
    for k in sorted({0, S - 1}):
        if precision == FP64:
            assert np.array_equal(x[:, k], want)
        else:
            assert norm_err(x[:, k], want) <= 1e-4


@pytest.mark.parametrize("S,precision", [(1, FP64), (96, FP32), (64, FP64)])
def test_autotune_picks_a_working_configuration(cuda, S, precision):
    from phdthesis_albertojimenezruiz_gb300.glu import autotune

    p = Plant(4, 8, 20)
    s = Symbolic(p.rowptr, p.colidx)
    ml, sc, ms = autotune(s, S, precision)
    assert sc in (SCHED_LEVELS, SCHED_PERSISTENT) and ms > 0
    num = Numeric(s, S, precision, sc, max_locals=ml)
    assert num.max_locals == ml
    o = O.Port(p.rowptr, p.colidx, s.array("perm_amd"))
    a, b = M.plant_batch(p, S, seed0=7, preset="c1")
    num.scatter(dev(pad_cols(a, num.ld)))
    num.refactor()
    x = dev(pad_cols(b, num.ld), np.float64 if precision == FP64 else np.float32)
    num.solve(x, original=True)
    x = x.cpu().numpy().reshape(s.n, num.ld)
    _, x_ref = o.scatter_refactor_solve(a[:, 0], b[:, 0])
    assert norm_err(x[:, 0], x_ref) <= (TOL64 if precision == FP64 else 1e-4)


@pytest.mark.parametrize("precision", [FP64, FP32])
@pytest.mark.parametrize("counts", [(1, 1, 1), (37, 64, 5)])
def test_group_of_size_classes_matches_members(cuda, precision, counts):
    """Three plant sizes refactored + solved by one launch per level give the
    same values as each handle alone (bit-identical: same arithmetic)."""
    import torch

    from phdthesis_albertojimenezruiz_gb300.glu import Group

    dims = [(2, 4, 10), (4, 8, 20), (3, 6, 12)]
    tdt = np.float64 if precision == FP64 else np.float32
    members, refs, xs = [], [], []
    for k, (d, S) in enumerate(zip(dims, counts)):
        p = Plant(*d)
        s = Symbolic(p.rowptr, p.colidx)
        a, b = M.plant_batch(p, S, seed0=50 + k, preset="c1")
        alone = Numeric(s, S, precision, SCHED_LEVELS)
        grouped = Numeric(s, S, precision, SCHED_LEVELS)
        for h in (alone, grouped):
            h.scatter(dev(pad_cols(a, h.ld)))
        xa = dev(pad_cols(b, alone.ld), tdt)
        alone.refactor()
        alone.solve(xa, original=True)
        torch.cuda.synchronize()
        refs.append((values_of(alone, int(s.nnz_lu)), xa.cpu().numpy(), int(s.nnz_lu)))
        members.append(grouped)
        xs.append(dev(pad_cols(b, grouped.ld), tdt))
    g = Group(members)
    g.refactor_solve(xs, original=True)
    torch.cuda.synchronize()
    for h, x, (lu_ref, x_ref, nnz), S in zip(members, xs, refs, counts):
        assert h.check()[0] == 0
        # padding columns (s >= S) hold no scenario
        assert np.array_equal(values_of(h, nnz)[:, :S], lu_ref[:, :S])
        assert np.array_equal(x.cpu().numpy().reshape(-1, h.ld)[:, :S],
                              x_ref.reshape(-1, h.ld)[:, :S])


def test_zero_pivot_reported_per_scenario(cuda):
    p = Plant(4, 8, 20)
    s = Symbolic(p.rowptr, p.colidx)
    S = 33
    a, b = M.plant_batch(p, S, seed0=5)
    bad = 17
    # zero every entry of one row in scenario `bad`: its pivot collapses
    row = int(s.array("row_orig")[0])
    a[p.rowptr[row]:p.rowptr[row + 1], bad] = 0.0
    for schedule in SCHEDULES:
        num = Numeric(s, S, FP64, schedule)
        num.scatter(dev(pad_cols(a, num.ld)))
        num.refactor()
        code, col, sc = num.check()
        assert code == N.OK + 3 and sc == bad, (code, col, sc)
        assert num.check() == (0, -1, -1)  # cleared
        # the other scenarios are unaffected
        o = O.Port(p.rowptr, p.colidx, s.array("perm_amd"))
        lu = values_of(num, int(s.nnz_lu))
        for k in (0, bad - 1, bad + 1, S - 1):
            lu_ref, _ = o.scatter_refactor_solve(a[:, k], b[:, k])
            assert rel_err(lu[:, k], lu_ref) <= TOL64


def test_host_dropin_entry_points(cuda):
    """pvglu_refactor_host / pvglu_solve_host: the reference's host-in,
    host-out semantics of factorize_electrical_system_CUDA and
    triangular_substitution_LU_CUDA."""
    g = load_golden("plant_c1")
    s = Symbolic(g["rowptr"], g["colidx"], g["perm_amd"])
    num = Numeric(s, 1, FP64)
    v = g["csc_in"].copy()
    num.refactor_host(v)
    assert rel_err(v, g["lu_seq"]) <= TOL64
    b = to_perm(g, g["b"])
    num.solve_host(b)
    assert norm_err(b, g["x_perm"]) <= TOL64


def test_scatter_refactor_solve_host_buffers(cuda):
    import torch

    p = Plant(10, 16, 20)
    s = Symbolic(p.rowptr, p.colidx)
    o = O.Port(p.rowptr, p.colidx, s.array("perm_amd"))
    S = 32
    a, b = M.plant_batch(p, S, seed0=900)
    num = Numeric(s, S, FP64, SCHED_PERSISTENT)
    a_h = torch.from_numpy(pad_cols(a, num.ld)).pin_memory()
    b_h = torch.from_numpy(pad_cols(b, num.ld)).pin_memory()
    x_h = torch.empty_like(b_h).pin_memory()
    stream = torch.cuda.current_stream()
    num.scatter_refactor_solve_host(a_h, b_h, x_h, stream=stream)
    stream.synchronize()
    x = x_h.numpy()
    for k in range(0, S, 5):
        _, x_ref = o.scatter_refactor_solve(a[:, k], b[:, k])
        assert norm_err(x[:, k], x_ref) <= TOL64


def test_barrier_timeout_is_reported_not_hung(cuda):
    code, ret = C.c_int(-1), C.c_int(-1)
    N.check(N.lib().pvglu_selftest_barrier_timeout(4, 20000, C.byref(code), C.byref(ret)),
            "selftest")
    assert code.value == 6  # PVGLU_ERR_BARRIER_TIMEOUT
    assert ret.value == 4   # every block returned
    # the context is still usable afterwards
    test_host_dropin_entry_points(cuda)


def test_loaded_symbolic_factors_bit_identical(cuda, tmp_path):
    """A handle built on a reloaded analysis computes the same FP64 factors
    and solutions as one built on the original."""
    p = Plant(4, 8, 20)
    s = Symbolic(p.rowptr, p.colidx)
    s.save(tmp_path / "s.pvs")
    t = Symbolic.load(tmp_path / "s.pvs")
    a, b = M.plant_batch(p, 40, seed0=3, preset="c1")
    out = []
    for sym in (s, t):
        num = Numeric(sym, 40, FP64, SCHED_LEVELS)
        num.scatter(dev(pad_cols(a, num.ld)))
        num.refactor()
        x = dev(pad_cols(b, num.ld))
        num.solve(x, original=True)
        out.append((values_of(num, int(sym.nnz_lu))[:, :40], x.cpu().numpy()[:, :40]))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_refinement_graph_matches_direct_launches(cuda):
    """The levels schedule replays the refinement from a graph with a
    conditional sweep loop, the persistent schedule launches it sweep by
    sweep: same solutions bit for bit, same sweep counts, also after the
    graph is rebuilt for new arguments and when the sweep cap stops it."""
    import torch

    p = Plant(10, 16, 20)
    s = Symbolic(p.rowptr, p.colidx)
    S = 96
    a, b = M.plant_batch(p, S, seed0=500, preset="c3")
    out = {}
    for sched in (SCHED_LEVELS, SCHED_PERSISTENT):
        num = Numeric(s, S, FP32, sched)
        a_dev = dev(pad_cols(a, num.ld))
        b_dev = dev(pad_cols(b, num.ld))
        num.scatter(a_dev)
        num.refactor()
        runs = []
        for tol, ms in ((1e-12, 8), (1e-12, 8), (1e-6, 8), (1e-300, 2), (1e-12, 1)):
            x = torch.full_like(b_dev, float("nan"))
            sweeps = torch.zeros(num.ld, dtype=torch.int32, device="cuda")
            num.solve_refined(a_dev, b_dev, x, tol=tol, max_sweeps=ms, sweeps=sweeps)
            torch.cuda.synchronize()
            runs.append((x.cpu().numpy()[:, :S], sweeps.cpu().numpy()[:S]))
        out[sched] = runs
    for (xg, sg), (xd, sd) in zip(out[SCHED_LEVELS], out[SCHED_PERSISTENT]):
        assert np.array_equal(sg, sd)
        assert np.array_equal(xg, xd)
    sw = [r[1] for r in out[SCHED_LEVELS]]
    assert (sw[0] > 1).all() and np.array_equal(sw[0], sw[1])
    assert (sw[2] <= sw[0]).all() and (sw[2] >= 1).all()
    assert (sw[3] == -1).all()
    assert (sw[4] == -1).all() or (sw[4] == 1).all()


_REFINE_SCRIPT = r"""
import sys
import numpy as np, torch
sys.path.insert(0, sys.argv[2])
import matrices as M
from phdthesis_albertojimenezruiz_gb300 import FP32, SCHED_LEVELS, Numeric, Plant, Symbolic
p = Plant(10, 16, 20)
s = Symbolic(p.rowptr, p.colidx)
S = 64
a, b = M.plant_batch(p, S, seed0=700, preset="c3")
num = Numeric(s, S, FP32, SCHED_LEVELS)
a_dev = torch.from_numpy(np.ascontiguousarray(a)).cuda()
b_dev = torch.from_numpy(np.ascontiguousarray(b)).cuda()
num.scatter(a_dev)
num.refactor()
x = torch.zeros_like(b_dev)
sw = torch.zeros(num.ld, dtype=torch.int32, device="cuda")
num.solve_refined(a_dev, b_dev, x, tol=1e-12, max_sweeps=8, sweeps=sw)
torch.cuda.synchronize()
np.save(sys.argv[1], np.concatenate([x.cpu().numpy().ravel(), sw.cpu().numpy().astype(np.float64)]))
"""


def test_refinement_profiling_switch_gives_the_same_bits(cuda, tmp_path):
    """PVGLU_REFINE_GRAPH=0 launches the refinement kernel by kernel instead
    of replaying the conditional graph: the results are bit-identical."""
    import os
    import subprocess
    import sys

    tests_dir = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(tests_dir)
    script = tmp_path / "refine.py"
    script.write_text(_REFINE_SCRIPT)
    outs = []
    for flag in ("1", "0"):
        out = tmp_path / f"x{flag}.npy"
        env = dict(os.environ, PVGLU_REFINE_GRAPH=flag, PYTHONPATH=root)
        subprocess.run([sys.executable, str(script), str(out), tests_dir], check=True, env=env,
                       cwd=root, timeout=600)
        outs.append(np.load(out))
    assert np.array_equal(outs[0], outs[1])


@pytest.mark.parametrize("schedule", [SCHED_LEVELS, SCHED_PERSISTENT])
def test_handles_with_different_table_sizes_coexist(cuda, schedule):
    """A handle with wide tables still launches after a handle with narrow
    tables was created (the kernels' shared-memory limit is process-wide),
    and both give the FP64 oracle's solution after refinement."""
    import torch

    p = Plant(10, 16, 20)
    s = Symbolic(p.rowptr, p.colidx)
    o = O.Port(p.rowptr, p.colidx, s.array("perm_amd"))
    S = 64
    a, b = M.plant_batch(p, S, seed0=900, preset="c3")
    wide = Numeric(s, S, FP32, schedule, max_locals=100)
    narrow = Numeric(s, S, FP32, schedule, max_locals=8)
    for num in (wide, narrow, wide):
        a_dev = dev(pad_cols(a, num.ld))
        b_dev = dev(pad_cols(b, num.ld))
        num.scatter(a_dev)
        num.refactor()
        x = torch.zeros_like(b_dev)
        num.solve_refined(a_dev, b_dev, x, tol=1e-12, max_sweeps=10)
        torch.cuda.synchronize()
        assert num.check()[0] == 0
        x = x.cpu().numpy()
        for k in (0, S - 1):
            _, x_ref = o.scatter_refactor_solve(a[:, k], b[:, k])
            assert np.abs(x[:, k] - x_ref).max() / np.abs(x_ref).max() <= 1e-10


def test_refine_residual_matches_numpy(cuda):
    """pvglu_refine_residual: r = b - J x with FP64 arithmetic, rounded to FP32,
    in pivot order (row p holds the residual of row row_orig[p])."""
    import torch

    p = Plant(4, 8, 20)
    s = Symbolic(p.rowptr, p.colidx)
    S = 64
    a, b = M.plant_batch(p, S, seed0=40, preset="c1")
    num = Numeric(s, S, FP32, SCHED_LEVELS)
    rng = np.random.default_rng(5)
    x = rng.uniform(-1.0, 1.0, (s.n, S)) * 30.0
    r = torch.full((s.n * num.ld,), float("nan"), dtype=torch.float32, device="cuda")
    num.refine_residual(dev(a), dev(b), dev(x), r)
    torch.cuda.synchronize()
    r = r.cpu().numpy().astype(np.float64).reshape(s.n, num.ld)[:, :S]
    row_orig = s.array("row_orig")
    got = np.empty_like(r)
    got[row_orig] = r
    rows = np.repeat(np.arange(s.n), np.diff(p.rowptr))
    for k in range(S):
        ax = np.zeros(s.n)
        np.add.at(ax, rows, a[:, k] * x[p.colidx, k])
        mag = np.zeros(s.n)
        np.add.at(mag, rows, np.abs(a[:, k] * x[p.colidx, k]))
        want = b[:, k] - ax
        assert np.all(np.abs(got[:, k] - want) <= 2.0 ** -23 * np.abs(want) + 1e-13 * (mag + np.abs(b[:, k])))


def test_refine_stamps_host_matches_oracle(cuda):
    """pvglu_refine_stamps_host: panel conductances and b from host memory,
    Jacobian from the registered stamps, x back in host memory, within 1e-10
    of the oracle's solve of the assembled Jacobian."""
    import torch

    p = Plant(4, 8, 20)
    s = Symbolic(p.rowptr, p.colidx)
    o = O.Port(p.rowptr, p.colidx, s.array("perm_amd"))
    S = 64
    g = np.stack([p.irradiance(seed=70 + k, preset="c1") for k in range(S)], axis=1)
    v = np.repeat(p.flat_start()[:, None], S, axis=1)
    a, b = p.companion_batch(g, v)
    _, didv = p.panel_iv(p.iph(g).ravel(), v.ravel())
    gpan = -didv.reshape(p.n_panels, S)
    num = Numeric(s, S, FP32, SCHED_LEVELS)
    num.set_stamps(p.n_panels, p.a_lin, p.contrib_ptr, p.contrib_panel, p.contrib_sign)
    g_h = torch.from_numpy(np.ascontiguousarray(gpan)).pin_memory()
    b_h = torch.from_numpy(np.ascontiguousarray(b)).pin_memory()
    x_h = torch.zeros_like(b_h).pin_memory()
    sw = torch.zeros(num.ld, dtype=torch.int32, device="cuda")
    num.refine_stamps_host(g_h, b_h, x_h, tol=1e-12, max_sweeps=10, sweeps=sw)
    torch.cuda.synchronize()
    assert (sw.cpu().numpy()[:S] > 0).all()
    x = x_h.numpy()
    for k in (0, 17, S - 1):
        _, x_ref = o.scatter_refactor_solve(a[:, k], b[:, k])
        assert np.abs(x[:, k] - x_ref).max() / np.abs(x_ref).max() <= 1e-10


def _values_bits(num: Numeric, count: int) -> np.ndarray:
    """The factor values' bit patterns, padding scenarios included."""
    import torch

    ts, it = ("<f8", np.uint64) if num.precision == FP64 else ("<f4", np.uint32)
    t = torch.as_tensor(_DevView(num.values_ptr(), (count * num.ld,), ts), device="cuda")
    torch.cuda.synchronize()
    return t.cpu().numpy().view(it).reshape(count, num.ld).copy()


@pytest.mark.parametrize("precision", [FP64, FP32])
@pytest.mark.parametrize("name,S,max_locals,merge,schedule", [
    ("plant_10x16x20", 37, 24, 1, SCHED_LEVELS),
    ("plant_10x16x20", 130, 8, 0, SCHED_LEVELS),
    ("plant_4x8x20", 64, 16, 2, SCHED_PERSISTENT),
    ("mesh_30x30", 64, 0, 2, SCHED_LEVELS),
    ("mesh_12x10", 64, 16, 1, SCHED_LEVELS),
    ("random_1500", 100, 0, 1, SCHED_LEVELS),
    ("block_1x20x20", 64, 24, 2, SCHED_LEVELS),
])
def test_scatter_refactor_one_pass_bit_identical(cuda, precision, name, S, max_locals, merge,
                                                 schedule):
    """pvglu_scatter_refactor reads each column's entries straight from A
    where the handle allows (batched, per-level schedule, no WIDE level) and
    falls back to scatter + refactor elsewhere (the persistent schedule; the
    reference-topology block plant, which has WIDE levels): the factors equal
    pvglu_scatter then pvglu_refactor bit for bit, padding scenarios
    included, after stale factors of other values were in the handle."""
    if name.startswith("plant_"):
        p = Plant(*map(int, name[6:].split("x")))
        s = Symbolic(p.rowptr, p.colidx)
        a, _ = M.plant_batch(p, S, seed0=70, preset="c3")
    elif name in M.CASES:
        rp, ci, a1, _ = M.CASES[name]()
        s = Symbolic(rp, ci)
        a = a1[:, None] * (1.0 + 1e-3 * np.arange(S))[None, :]
    else:
        g = load_golden(name)
        s = Symbolic(g["rowptr"], g["colidx"], g["perm_amd"])
        a = g["a"][:, None] * (1.0 + 1e-3 * np.arange(S))[None, :]
    t = {"max_locals": max_locals, "wide_threshold": 0, "merge_chains": merge,
         "schedule": schedule}
    ref = Numeric(s, S, precision, tuning=t)
    a_dev = dev(pad_cols(a, ref.ld))
    ref.scatter(a_dev)
    ref.refactor()
    assert ref.check()[0] == 0
    want = _values_bits(ref, int(s.nnz_lu))
    one = Numeric(s, S, precision, tuning=t)
    one.scatter(dev(pad_cols(a[:, ::-1] * 3.0, one.ld)))
    one.refactor()
    one.check()
    one.scatter_refactor(a_dev)
    assert one.check()[0] == 0
    assert np.array_equal(_values_bits(one, int(s.nnz_lu)), want)


@pytest.mark.parametrize("precision", [FP64, FP32])
def test_scatter_refactor_reports_zero_pivot(cuda, precision):
    """A zero pivot in one scenario: the one-pass scatter + refactor reports
    the same column and scenario as pvglu_scatter + pvglu_refactor."""
    p = Plant(4, 8, 20)
    s = Symbolic(p.rowptr, p.colidx)
    S = 33
    a, _ = M.plant_batch(p, S, seed0=5)
    row = int(s.array("row_orig")[0])
    a[p.rowptr[row]:p.rowptr[row + 1], 17] = 0.0
    got = []
    for one_pass in (False, True):
        num = Numeric(s, S, precision, SCHED_LEVELS)
        a_dev = dev(pad_cols(a, num.ld))
        if one_pass:
            num.scatter_refactor(a_dev)
        else:
            num.scatter(a_dev)
            num.refactor()
        got.append(num.check())
    assert got[0] == got[1] and got[0][0] == N.OK + 3 and got[0][2] == 17, got


@pytest.mark.parametrize("precision,parts", [(FP32, 4), (FP64, 2)])
def test_blocks_match_one_handle(cuda, precision, parts):
    """pvglu_blocks: the scenarios split into blocks on streams of their own
    give, block by block, the same solutions (and refinement sweeps) as one
    handle over all of them, bit for bit."""
    import torch

    from phdthesis_albertojimenezruiz_gb300 import Blocks

    p = Plant(10, 16, 20)
    s = Symbolic(p.rowptr, p.colidx)
    S = 256
    a, b = M.plant_batch(p, S, seed0=1200, preset="c3")
    one = Numeric(s, S, precision, SCHED_LEVELS)
    a_dev, b_dev = dev(pad_cols(a, one.ld)), dev(pad_cols(b, one.ld))
    x_one = torch.zeros_like(b_dev)
    sw_one = torch.zeros(one.ld, dtype=torch.int32, device="cuda")
    one.scatter_refactor(a_dev)
    if precision == FP32:
        one.solve_refined(a_dev, b_dev, x_one, tol=1e-12, max_sweeps=8, sweeps=sw_one)
    else:
        x_one.copy_(b_dev)
        one.solve(x_one, original=True)
    torch.cuda.synchronize()
    blk = Blocks(s, S, parts, precision)
    H = S // parts
    a_k = [dev(pad_cols(a[:, k * H:(k + 1) * H], blk.parts[k].ld)) for k in range(parts)]
    b_k = [dev(pad_cols(b[:, k * H:(k + 1) * H], blk.parts[k].ld)) for k in range(parts)]
    x_k = [torch.full_like(t, float("nan")) for t in b_k]
    sw_k = [torch.zeros(blk.parts[k].ld, dtype=torch.int32, device="cuda") for k in range(parts)]
    stream = torch.cuda.Stream()
    blk.step(a_k, b_k, x_k, tol=1e-12, max_sweeps=8, sweeps=sw_k, stream=stream)
    stream.synchronize()
    # Unjoined steps, each block running on: the same after a join.
    for _ in range(2):
        blk.step(a_k, b_k, x_k, tol=1e-12, max_sweeps=8, sweeps=sw_k, stream=stream, join=False)
    blk.join(stream)
    stream.synchronize()
    for k in range(parts):
        assert blk.parts[k].check()[0] == 0
        got = x_k[k].cpu().numpy()[:, :H]
        want = x_one.cpu().numpy()[:, k * H:(k + 1) * H]
        assert np.array_equal(got, want), k
        if precision == FP32:
            assert np.array_equal(sw_k[k].cpu().numpy()[:H],
                                  sw_one.cpu().numpy()[k * H:(k + 1) * H]), k
