"""Newton driver and adjoint (include/pvglu_newton.h) against the CPU oracle's
restatement of the simulator's Newton loop (oracle/oracle_newton.cpp).

CPU tests pin the oracle itself: the panel law against an independent
bisection of the implicit single-diode equation, the converged operating
point against Kirchhoff's current law with the true element currents, and
the oracle's adjoint against central finite differences of full Newton
solves.  GPU tests run the device driver through the C ABI.

Tolerances: FP64 voltages and node solutions bit-identical with equal
iteration counts (the panel law uses its own exp/log and no multiply-add
contraction on either side, and the GLU is the reference's arithmetic);
FP32 factors + FP64 refinement 1e-10 normwise relative (conftest.norm_err);
adjoint 1e-10 against the oracle's adjoint and 1e-6 against central
differences (step 1e-2 W/m^2, truncation ~1e-7).
"""
from __future__ import annotations

import numpy as np
import pytest
from conftest import norm_err

from oracle import oracle as O
from phdthesis_albertojimenezruiz_gb300 import (FP32, FP64, GMIN_STAGES, SCHED_LEVELS,
                                                SCHED_PERSISTENT, SCHED_THREAD_CHAIN, Newton,
                                                Numeric, Plant, Symbolic)
from phdthesis_albertojimenezruiz_gb300 import _native as N

SCHEDULES = [SCHED_LEVELS, SCHED_PERSISTENT, SCHED_THREAD_CHAIN]
G_TO_IPH = 8.5 / 1000.0  # Iph = 8.5 A at 1000 W/m^2


def bright(p: Plant, seed: int) -> np.ndarray:
    """Irradiance with per-panel variation 400-1000 W/m^2 (every panel lit)."""
    return 1000.0 - np.random.default_rng(seed).uniform(0.0, 600.0, p.n_panels)


def objective(p: Plant) -> np.ndarray:
    """P = power into the MPPT sinks = -V_mppt * sum of source currents."""
    d = np.zeros(p.n)
    d[p.inv_current] = -p.v_mppt
    return d


def setup(dims):
    p = Plant(*dims)
    sym = Symbolic(p.rowptr, p.colidx)
    port = O.Port(p.rowptr, p.colidx, sym.array("perm_amd"))
    return p, sym, port


def kcl_residual(p: Plant, iph: np.ndarray, x: np.ndarray) -> float:
    vx = np.where(p.pan_hi >= 0, x[np.maximum(p.pan_hi, 0)], 0.0) - \
        np.where(p.pan_lo >= 0, x[np.maximum(p.pan_lo, 0)], 0.0)
    cur, _ = p.panel_iv(iph, vx)
    F = -p.b_lin.copy()
    rows = np.repeat(np.arange(p.n), np.diff(p.rowptr))
    np.add.at(F, rows, p.a_lin * x[p.colidx])
    hi, lo = p.pan_hi >= 0, p.pan_lo >= 0
    np.add.at(F, p.pan_hi[hi], -cur[hi])
    np.add.at(F, p.pan_lo[lo], cur[lo])
    return float(np.abs(F).max())


# --------------------------------------------------------------------------
# CPU: the oracle pinned by physics and finite differences


def test_panel_exp_log_accuracy():
    import ctypes as C

    rng = np.random.default_rng(0)
    x = np.concatenate([rng.uniform(-745, 709, 50000), rng.uniform(-1, 1, 50000),
                        [0.0, 1.0, -1.0, 700.0, -700.0]])
    e = np.empty_like(x)
    N.check(N.lib().pvglu_plant_exp_log(len(x), C.c_void_p(x.ctypes.data),
                                        C.c_void_p(e.ctypes.data), None), "exp")
    ref = np.exp(x)
    ok = ref > 2.3e-308
    assert np.max(np.abs(e[ok] - ref[ok]) / np.spacing(ref[ok])) <= 2.0
    xs = np.concatenate([10 ** rng.uniform(-300, 300, 50000), rng.uniform(0.5, 2.0, 50000),
                         [1.0, 2.0, 0.5, 1e-310]])
    lg = np.empty_like(xs)
    N.check(N.lib().pvglu_plant_exp_log(len(xs), C.c_void_p(xs.ctypes.data), None,
                                        C.c_void_p(lg.ctypes.data)), "log")
    ref = np.log(xs)
    nz = ref != 0
    assert lg[xs == 1.0][0] == 0.0
    assert np.max(np.abs(lg[nz] - ref[nz]) / np.spacing(np.abs(ref[nz]))) <= 4.0


def test_panel_law_matches_bisection():
    p = Plant(1, 1, 3)
    i = p.info
    rng = np.random.default_rng(3)
    v = np.concatenate([rng.uniform(-120, 60, 400), [0.0, p.voc_panel]])
    iph = rng.uniform(0.0, 9.0, len(v))
    cur, didv = p.panel_iv(iph, v)
    # Independent: bisection on the diode voltage vd of
    #   (vd - V)/Rs = Iph - I0 (exp(vd/a) - 1) - vd/Rsh   (strictly decreasing in vd)
    i0, a, rs, rsh = i["panel_i0"], i["panel_a"], i["panel_rs"], i["panel_rsh"]
    h = lambda vd: iph + i0 - i0 * np.exp(vd / a) - vd / rsh - (vd - v) / rs  # noqa: E731
    lo = np.minimum(v, 0.0) - 1e3
    hi = np.full_like(v, 80.0)
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        pos = h(mid) > 0
        lo = np.where(pos, mid, lo)
        hi = np.where(pos, hi, mid)
    vd = 0.5 * (lo + hi)
    ref = (vd - v) / rs
    assert np.max(np.abs(cur - ref) / np.maximum(np.abs(ref), 1e-3)) < 1e-10
    gd = i0 / a * np.exp(vd / a) + 1.0 / rsh
    assert np.max(np.abs(didv + gd / (1 + rs * gd)) / (gd / (1 + rs * gd))) < 1e-9


@pytest.mark.parametrize("dims", [(1, 2, 5), (2, 4, 10)])
def test_oracle_newton_satisfies_kcl(dims):
    p, sym, port = setup(dims)
    iph = p.iph(bright(p, 1))
    rc, it, diff, v, x = port.newton(p, iph, p.flat_start(), GMIN_STAGES, 1e-9)
    assert rc == 0 and 10 < it < 5000 and diff < 1e-9
    assert kcl_residual(p, iph, x) < 1e-8 * np.abs(x).max()
    assert objective(p) @ x > 0  # the plant delivers power


def test_oracle_newton_iteration_cap_and_stage_tolerance():
    p, sym, port = setup((1, 2, 5))
    iph = p.iph(bright(p, 2))
    rc, it, _, _, _ = port.newton(p, iph, p.flat_start(), GMIN_STAGES, 1e-9, max_iterations=7)
    assert rc == 2 and it == 7
    # Reference tolerance 1e-6 * n stops earlier than 1e-9.
    _, it_loose, *_ = port.newton(p, iph, p.flat_start(), GMIN_STAGES, 1e-6 * p.n)
    _, it_tight, *_ = port.newton(p, iph, p.flat_start(), GMIN_STAGES, 1e-9)
    assert it_loose < it_tight


@pytest.mark.parametrize("dims", [(1, 2, 5), (2, 4, 10)])
def test_oracle_adjoint_matches_finite_differences(dims):
    p, sym, port = setup(dims)
    g = bright(p, 1)
    dpdx = objective(p)

    def solve(gg):
        rc, _, _, v, x = port.newton(p, p.iph(gg), p.flat_start(), GMIN_STAGES, 1e-9)
        assert rc == 0
        return v, x

    v, _ = solve(g)
    adj = port.adjoint(p, p.iph(g), v, dpdx) * G_TO_IPH
    h = 1e-2
    # A direction without sign changes keeps the derivative away from cancellation.
    d = np.random.default_rng(5).uniform(0.5, 1.0, p.n_panels)
    fd = (dpdx @ solve(g + h * d)[1] - dpdx @ solve(g - h * d)[1]) / (2 * h)
    assert abs(adj @ d - fd) <= 1e-6 * abs(fd)
    # One panel: the most sensitive one (a near-zero derivative would measure
    # the finite-difference noise, ~1e-8 W per W/m^2, instead).
    k = int(np.argmax(np.abs(adj)))
    e = np.zeros(p.n_panels)
    e[k] = 1.0
    fd_k = (dpdx @ solve(g + h * e)[1] - dpdx @ solve(g - h * e)[1]) / (2 * h)
    assert abs(adj[k] - fd_k) <= 1e-6 * abs(fd_k)


def test_inverter_blocks_are_the_one_inverter_plant():
    """Block v of a multi-inverter plant (pattern, linear values, panel
    terminals, sources) is Plant(1, strings, series) shifted by v blocks, with
    no entry outside the diagonal blocks: the plant decomposes by inverter."""
    p = Plant(3, 4, 6)
    q = Plant(1, 4, 6)
    rows = np.repeat(np.arange(p.n), np.diff(p.rowptr))
    for v in range(3):
        nodes, pans = p.inverter_block(v)
        off = nodes.start
        sel = (rows >= nodes.start) & (rows < nodes.stop)
        assert (p.colidx[sel] >= nodes.start).all() and (p.colidx[sel] < nodes.stop).all()
        sub_ptr = p.rowptr[nodes.start:nodes.stop + 1] - p.rowptr[nodes.start]
        assert np.array_equal(sub_ptr, q.rowptr)
        assert np.array_equal(p.colidx[sel] - off, q.colidx)
        assert np.array_equal(p.a_lin[sel], q.a_lin)
        assert np.array_equal(p.b_lin[nodes], q.b_lin)
        shift = lambda a: np.where(a >= 0, a - off, -1)  # noqa: E731
        assert np.array_equal(shift(p.pan_hi[pans]), q.pan_hi)
        assert np.array_equal(shift(p.pan_lo[pans]), q.pan_lo)
        assert p.inv_current[v] - off == q.inv_current[0]


def test_extended_precision_differences_match_oracle_adjoint():
    """The extended-precision central difference (oracle_fd_ext) reproduces
    the oracle's FP64 adjoint per panel to 1e-6 at the configuration's step
    of 1e-3 W/m^2, where FP64 differences of full Newton solves cannot (node
    voltages near 1 kV are quantised at 2e-13 V)."""
    p, sym, port = setup((1, 6, 12))
    g = bright(p, 3)
    rc, _, _, v, _ = port.newton(p, p.iph(g), p.flat_start(), GMIN_STAGES, 1e-9)
    assert rc == 0
    dpdx = objective(p)
    adj = port.adjoint(p, p.iph(g), v, dpdx) * G_TO_IPH
    h = 1e-3
    for k in np.random.default_rng(11).choice(p.n_panels, 12, replace=False):
        fd, its, res = port.fd_ext(p, p.iph(g), v, dpdx, int(k), G_TO_IPH * h)
        assert abs(G_TO_IPH * fd - adj[k]) <= 1e-6 * abs(adj[k]), (k, fd, adj[k], its, res)


# --------------------------------------------------------------------------
# GPU: the device driver through the C ABI


def dev(a, dtype=np.float64):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).cuda()


def cols(a: np.ndarray, ld: int) -> np.ndarray:
    """[rows, S] -> [rows, ld] (padding columns zero); 1-D = one scenario."""
    a = a.reshape(a.shape[0], -1)
    out = np.zeros((a.shape[0], ld))
    out[:, : a.shape[1]] = a
    return out


def run_device(p, sym, g_cols, precision, schedule, tol, max_iterations=5000, check_every=4):
    """Device Newton for the scenarios in g_cols [n_panels, S]."""
    import torch

    S = g_cols.shape[1]
    num = Numeric(sym, S, precision, schedule)
    nw = Newton.for_plant(num, p)
    ld = num.ld
    nw.set_iph(dev(cols(p.iph(g_cols), ld)))
    nw.set_voltages(dev(cols(np.repeat(p.flat_start()[:, None], S, 1), ld)))
    nw.run(tol, max_iterations=max_iterations, check_every=check_every)
    it, out, diff = nw.results()
    x = torch.zeros(p.n * ld, dtype=torch.float64, device="cuda")
    nw.solution(x)
    vt = torch.as_tensor(_DevView(nw.voltages_ptr(), (p.n_panels * ld,)), device="cuda")
    torch.cuda.synchronize()
    x = x.cpu().numpy().reshape(p.n, ld)[:, :S]
    v = vt.cpu().numpy().reshape(p.n_panels, ld)[:, :S]
    return num, nw, it, out, diff, v, x


class _DevView:
    def __init__(self, ptr, shape):
        self.__cuda_array_interface__ = {"shape": shape, "typestr": "<f8",
                                         "data": (ptr, False), "version": 3}


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [FP64, FP32])
def test_scatter_stamps_equals_explicit_values(cuda, precision):
    import torch

    from test_gpu_parity import values_of

    p, sym, _ = setup((2, 4, 10))
    S = 3
    num = Numeric(sym, S, precision, SCHED_LEVELS)
    Newton.for_plant(num, p)  # registers the stamps
    ld = num.ld
    rng = np.random.default_rng(0)
    gel = rng.uniform(0.01, 2.0, (p.n_panels, S))
    gmin = np.array([0.0, 0.5, 100.0])
    num.scatter_stamps(dev(cols(gel, ld)), dev(np.pad(gmin, (0, ld - S))))
    stamped = values_of(num, int(sym.nnz_lu))
    # Same additions in the same order on the host: base, then per element
    # in element order +-G and, if positive, +-gmin.
    a = np.repeat(p.a_lin[:, None], S, 1)
    ptr = p.contrib_ptr
    for e in range(len(p.a_lin)):
        for c in range(ptr[e], ptr[e + 1]):
            sg = float(p.contrib_sign[c])
            for s in range(S):
                a[e, s] = a[e, s] + sg * gel[p.contrib_panel[c], s]
                if gmin[s] > 0:
                    a[e, s] = a[e, s] + sg * gmin[s]
    num.scatter(dev(cols(a, ld)))
    explicit = values_of(num, int(sym.nnz_lu))
    assert np.array_equal(stamped, explicit)
    torch.cuda.synchronize()


@pytest.mark.gpu
@pytest.mark.parametrize("schedule", SCHEDULES)
@pytest.mark.parametrize("dims,S", [((2, 4, 10), 1), ((1, 8, 20), 3)])
def test_newton_fp64_matches_oracle(cuda, dims, S, schedule):
    p, sym, port = setup(dims)
    g = np.stack([bright(p, 10 + s) for s in range(S)], 1)
    tol = 1e-6 * p.n
    num, nw, it, out, diff, v, x = run_device(p, sym, g, FP64, schedule, tol)
    assert num.check()[0] == 0
    for s in range(S):
        rc, it_o, diff_o, v_o, x_o = port.newton(p, p.iph(g[:, s]), p.flat_start(),
                                                 GMIN_STAGES, tol)
        assert rc == 0 and out[s] == N.NEWTON_CONVERGED
        assert it[s] == it_o
        assert np.array_equal(v[:, s], v_o), norm_err(v[:, s], v_o)
        assert np.array_equal(x[:, s], x_o), norm_err(x[:, s], x_o)
    if schedule == SCHED_LEVELS:
        assert nw.last_run()[1], "iteration body did not run as a CUDA graph"


@pytest.mark.gpu
@pytest.mark.parametrize("schedule", [SCHED_LEVELS, SCHED_PERSISTENT])
def test_newton_fp32_refined_matches_oracle(cuda, schedule):
    p, sym, port = setup((2, 4, 10))
    S = 3
    g = np.stack([bright(p, 20 + s) for s in range(S)], 1)
    tol = 1e-9
    num, nw, it, out, diff, v, x = run_device(p, sym, g, FP32, schedule, tol)
    for s in range(S):
        rc, it_o, _, v_o, x_o = port.newton(p, p.iph(g[:, s]), p.flat_start(), GMIN_STAGES, tol)
        assert rc == 0 and out[s] == N.NEWTON_CONVERGED
        # The refined linear solves stop at an estimated 1e-12, so the damped
        # iteration may take a few iterations more or less than FP64.
        assert abs(int(it[s]) - it_o) <= max(3, it_o // 20)
        assert norm_err(v[:, s], v_o) <= 1e-10
        assert norm_err(x[:, s], x_o) <= 1e-10


@pytest.mark.gpu
def test_newton_iteration_cap(cuda):
    p, sym, _ = setup((1, 2, 5))
    g = bright(p, 3)[:, None]
    _, nw, it, out, _, _, _ = run_device(p, sym, g, FP64, SCHED_LEVELS, 1e-9, max_iterations=7,
                                         check_every=3)
    assert it[0] == 7 and out[0] == N.NEWTON_MAX_ITERATIONS
    assert nw.last_run()[0] <= 7 + 3


@pytest.mark.gpu
def test_newton_bad_arguments(cuda):
    p, sym, _ = setup((1, 2, 5))
    num = Numeric(sym, 1, FP64)
    nw = Newton.for_plant(num, p)
    with pytest.raises(N.PvgluError):
        nw.run(1e-6, gmin=[])
    with pytest.raises(N.PvgluError):
        nw.run(1e-6, gmin=list(range(17)))
    with pytest.raises(N.PvgluError):
        nw.run(0.0)
    with pytest.raises(N.PvgluError):  # a terminal outside the pattern's unknowns
        Newton(num, 1, [p.n], [-1], p.a_lin, p.b_lin, 1e-9, 2.0, 0.3, 300.0)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [FP64, FP32])
def test_adjoint_matches_oracle_and_finite_differences(cuda, precision):
    import torch

    p, sym, port = setup((2, 4, 10))
    g0 = bright(p, 1)
    h = 1e-2
    d = np.random.default_rng(5).uniform(0.5, 1.0, p.n_panels)
    g = np.stack([g0, g0 + h * d, g0 - h * d], 1)
    num, nw, it, out, diff, v, x = run_device(p, sym, g, precision, SCHED_PERSISTENT, 1e-9)
    assert (out == N.NEWTON_CONVERGED).all()
    dpdx = objective(p)
    ld = num.ld
    dpdiph = torch.zeros(p.n_panels * ld, dtype=torch.float64, device="cuda")
    nw.adjoint(dev(cols(np.repeat(dpdx[:, None], 3, 1), ld)), dpdiph)
    torch.cuda.synchronize()
    adj = dpdiph.cpu().numpy().reshape(p.n_panels, ld)[:, 0]
    ref = port.adjoint(p, p.iph(g0), v[:, 0], dpdx)
    assert norm_err(adj, ref) <= (1e-10 if precision == FP64 else 1e-8)
    fd = (dpdx @ x[:, 1] - dpdx @ x[:, 2]) / (2 * h)
    assert abs(G_TO_IPH * adj @ d - fd) <= 1e-6 * abs(fd)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [FP64, FP32])
def test_adjoint_per_panel_vs_extended_central_differences(cuda, precision):
    """Per-panel dP/dG from the device adjoint at the device's converged
    operating point against central differences at h = 1e-3 W/m^2 on 20
    random panels, each difference solved in extended precision on the
    panel's inverter block (the plant decomposes by inverter): 1e-6
    relative per panel, in both forward modes."""
    import torch

    p, sym, port = setup((3, 8, 20))
    g0 = bright(p, 7)
    num, nw, it, out, diff, v, x = run_device(p, sym, g0[:, None], precision, SCHED_LEVELS,
                                             1e-9)
    assert (out == N.NEWTON_CONVERGED).all()
    dpdx = objective(p)
    ld = num.ld
    dpdiph = torch.zeros(p.n_panels * ld, dtype=torch.float64, device="cuda")
    nw.adjoint(dev(cols(dpdx, ld)), dpdiph)
    torch.cuda.synchronize()
    adj = G_TO_IPH * dpdiph.cpu().numpy().reshape(p.n_panels, ld)[:, 0]
    q = Plant(1, 8, 20)
    qs = Symbolic(q.rowptr, q.colidx)
    qport = O.Port(q.rowptr, q.colidx, qs.array("perm_amd"))
    iph = p.iph(g0)
    h = 1e-3
    for k in np.random.default_rng(13).choice(p.n_panels, 20, replace=False):
        inv = int(k) // (8 * 20)
        nodes, pans = p.inverter_block(inv)
        fd, its, res = qport.fd_ext(q, iph[pans], v[pans, 0], objective(q), int(k) - pans.start,
                                    G_TO_IPH * h)
        assert abs(G_TO_IPH * fd - adj[k]) <= 1e-6 * abs(adj[k]), (k, G_TO_IPH * fd, adj[k])


@pytest.mark.gpu
def test_refine_transposed_and_stamped(cuda):
    import torch

    p, sym, port = setup((2, 4, 10))
    S = 2
    rng = np.random.default_rng(9)
    gel = rng.uniform(0.01, 1.0, (p.n_panels, S))
    num = Numeric(sym, S, FP32, SCHED_LEVELS)
    Newton.for_plant(num, p)
    ld = num.ld
    gd = dev(cols(gel, ld))
    num.scatter_stamps(gd)
    num.refactor()
    b = rng.standard_normal((p.n, S))
    xt = torch.zeros(p.n * ld, dtype=torch.float64, device="cuda")
    num.refine(dev(cols(b, ld)), xt, g=gd, transpose=True, tol=1e-13, max_sweeps=12)
    torch.cuda.synchronize()
    xt = xt.cpu().numpy().reshape(p.n, ld)
    for s in range(S):
        a = p.jacobian_values(gel[:, s])
        A = np.zeros((p.n, p.n))
        rows = np.repeat(np.arange(p.n), np.diff(p.rowptr))
        np.add.at(A, (rows, p.colidx), a)
        ref = np.linalg.solve(A.T, b[:, s])
        assert norm_err(xt[:, s], ref) <= 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("preset", ["c1", "c4"])
def test_device_irradiance_field_matches_host(cuda, preset):
    """The device field gives the host generator's irradiance bit for bit at
    every time step, and a Newton solve fed from it matches one fed with the
    host photocurrents."""
    import torch

    p, sym, port = setup((2, 4, 10))
    S = 3
    seeds = [11, 12, 13]
    num = Numeric(sym, S, FP64, SCHED_LEVELS)
    nw = Newton.for_plant(num, p)
    ld = num.ld
    nw.set_field(p.pan_x, p.pan_y, [p.shadows(sd, preset) for sd in seeds],
                 iph_per_g=p.info["iph_stc"] / 1000.0)
    g_dev = torch.zeros(p.n_panels * ld, dtype=torch.float64, device="cuda")
    for t in (0.0, 1.0, 7.5):
        nw.field_iph(t, g_dev)
        torch.cuda.synchronize()
        got = g_dev.cpu().numpy().reshape(p.n_panels, ld)[:, :S]
        want = np.stack([p.irradiance(sd, t, preset) for sd in seeds], 1)
        assert np.array_equal(got, want), t
    # Newton from the field at t = 7.5 vs from host photocurrents.
    v0 = dev(cols(np.repeat(p.flat_start()[:, None], S, 1), ld))
    nw.set_voltages(v0)
    nw.run(1e-6 * p.n)
    x1 = torch.zeros(p.n * ld, dtype=torch.float64, device="cuda")
    nw.solution(x1)
    nw.set_iph(dev(cols((p.info["iph_stc"] / 1000.0) * want, ld)))  # the field's product order
    nw.set_voltages(v0)
    nw.run(1e-6 * p.n)
    x2 = torch.zeros(p.n * ld, dtype=torch.float64, device="cuda")
    nw.solution(x2)
    torch.cuda.synchronize()
    assert np.array_equal(x1.cpu().numpy(), x2.cpu().numpy())


@pytest.mark.gpu
def test_kirchhoff_mismatch_after_convergence(cuda):
    """The device mismatch agrees with a host evaluation of Kirchhoff's law
    on the same node solution, and is below 1e-9 A once the iteration has
    converged to a tight tolerance (the convergence test of the synthetic
    configurations)."""
    p, sym, port = setup((4, 8, 20))
    S = 2
    g = np.stack([bright(p, 30 + s) for s in range(S)], 1)
    # 1e-9 on the summed |dV| of 640 panels sits just above the rounding floor
    num, nw, it, out, diff, v, x = run_device(p, sym, g, FP64, SCHED_LEVELS, 1e-9)
    assert (out == N.NEWTON_CONVERGED).all()
    mm = nw.mismatch()
    for s in range(S):
        host = kcl_residual(p, p.iph(g[:, s]), x[:, s])
        assert abs(mm[s] - host) <= 1e-12 + 1e-6 * host
        assert mm[s] < 1e-9


@pytest.mark.gpu
def test_plant_power_autograd(cuda):
    """plant_power: forward = device Newton, backward = adjoint; the autograd
    gradient equals the oracle's adjoint and a central difference."""
    import torch

    from phdthesis_albertojimenezruiz_gb300 import plant_power

    p, sym, port = setup((2, 4, 10))
    S = 2
    g0 = np.stack([bright(p, 40 + s) for s in range(S)], 1)
    num = Numeric(sym, S, FP64, SCHED_LEVELS)
    nw = Newton.for_plant(num, p)
    g = torch.tensor(g0, device="cuda", requires_grad=True)
    P = plant_power(nw, p, g)
    P.sum().backward()
    grad = g.grad.cpu().numpy()
    v = torch.as_tensor(_DevView(nw.voltages_ptr(), (p.n_panels * num.ld,)),
                        device="cuda").cpu().numpy().reshape(p.n_panels, num.ld)
    for s in range(S):
        ref = port.adjoint(p, p.iph(g0[:, s]), v[:, s], objective(p)) * G_TO_IPH
        assert norm_err(grad[:, s], ref) <= 1e-10
    h = 1e-2
    d = np.random.default_rng(2).uniform(0.5, 1.0, p.n_panels)
    with torch.no_grad():
        up = plant_power(nw, p, torch.tensor(g0 + h * d[:, None], device="cuda"))
        dn = plant_power(nw, p, torch.tensor(g0 - h * d[:, None], device="cuda"))
    fd = ((up - dn) / (2 * h)).cpu().numpy()
    assert np.all(np.abs(grad.T @ d - fd) <= 1e-6 * np.abs(fd))


@pytest.mark.gpu
@pytest.mark.parametrize("schedule", [SCHED_LEVELS, SCHED_PERSISTENT])
def test_broken_panels_match_oracle(cuda, schedule):
    """Broken panels become 1e-5 ohm wires on the same pattern (no new
    analysis): the device Newton and adjoint equal the oracle's."""
    import torch

    p, sym, port = setup((2, 4, 10))
    S = 2
    g = np.stack([bright(p, 50 + s) for s in range(S)], 1)
    broken = np.zeros(p.n_panels, np.int32)
    broken[[3, 17, 41]] = 1
    num = Numeric(sym, S, FP64, schedule)
    nw = Newton.for_plant(num, p)
    nw.set_broken(broken)
    ld = num.ld
    nw.set_iph(dev(cols(p.iph(g), ld)))
    nw.set_voltages(dev(cols(np.repeat(p.flat_start()[:, None], S, 1), ld)))
    tol = 1e-6 * p.n
    nw.run(tol)
    it, out, _ = nw.results()
    x = torch.zeros(p.n * ld, dtype=torch.float64, device="cuda")
    nw.solution(x)
    dpdx = objective(p)
    grad = torch.zeros(p.n_panels * ld, dtype=torch.float64, device="cuda")
    v = torch.as_tensor(_DevView(nw.voltages_ptr(), (p.n_panels * ld,)),
                        device="cuda").cpu().numpy().reshape(p.n_panels, ld)
    nw.adjoint(dev(cols(np.repeat(dpdx[:, None], S, 1), ld)), grad)
    torch.cuda.synchronize()
    x = x.cpu().numpy().reshape(p.n, ld)
    grad = grad.cpu().numpy().reshape(p.n_panels, ld)
    for s in range(S):
        rc, it_o, _, v_o, x_o = port.newton(p, p.iph(g[:, s]), p.flat_start(), GMIN_STAGES, tol,
                                            broken=broken)
        assert rc == 0 and out[s] == N.NEWTON_CONVERGED and it[s] == it_o
        assert np.array_equal(x[:, s], x_o)
        ref = port.adjoint(p, p.iph(g[:, s]), v[:, s], dpdx, broken=broken)
        assert norm_err(grad[:, s], ref) <= 1e-10
        assert np.all(grad[broken == 1, s] == 0.0)
