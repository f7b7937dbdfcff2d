"""Benchmark: refactor+solve/s on the ~35k-unknown PV plant Jacobian.

Workload (one "step" = one pass of the hot path over one batch): the
50 x 24 x 28 plant (inverters x strings x series panels, 33,750 unknowns),
S scenarios with seeded Gaussian-shadow irradiance fields (5 shadows),
companion Jacobians at the flat start.  Each step scatters the FP64 Jacobian
values into the filled pattern, refactorizes in FP32 and solves with FP64
iterative refinement until every scenario reaches max|dx| <= 1e-12 max|x|
(which puts the solution within 1e-10 of the FP64 solution).  The S
scenarios run as --blocks scenario blocks side by side, each on a stream of
its own (pvglu_blocks_step; one handle of all S is timed beside it as
`single_handle`).  `value` counts
refactor+solves (scenarios) per second with inputs resident in HBM; `e2e` is
the same through the host-buffer C-ABI call (H2D of A and b, D2H of x every
step).  The plain single-instance FP64 GPU path (scatter + refactor + solve,
one launch per level) is measured beside it.

--impl reference times the reference's own CPU GLU path (level-ordered GLU
+ CSC substitution, GLU_CSC_CPU_levels_strings.cpp / GLU_CSC_CPU_Triangular.cpp)
on the host cores: the reference build in oracle/_ref where it exists, else
the oracle's restatement of it.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

DIMS = (50, 24, 28)
METRIC = "refactor+solve/s, 35k-unknown PV Jacobian: batched+FP32-IR vs plain FP64 GPU"
UNIT = "refactor+solve/s"
IR_TOL = 1e-12
REFACTOR_TRAFFIC_512 = 610.6e6  # bytes, ncu dram__bytes_read.sum + dram__bytes_write.sum
RESIDUAL_TRAFFIC_512 = 735.3e6  # bytes, the same for one k_residual_rows launch
IR_MAX_SWEEPS = 6
# The headline's 512 scenarios as 4 blocks of 128 on 4 streams (pvglu_blocks):
# measured per step 1 / 2 / 4 / 8 blocks 1.010 / 1.006 / 0.960 / 0.989 ms.
HEADLINE_BLOCKS = 4


_TUNED: dict = {}


def _autotune(sym, S: int, precision: int):
    """pvglu_autotune_ex, once per pattern, scenario count and precision in
    this process (several sections use the same handles)."""
    from phdthesis_albertojimenezruiz_gb300.glu import autotune_ex

    key = (sym.n, int(sym.nnz_a), int(sym.nnz_lu), sym.info["lu_levels"], S, precision)
    if key not in _TUNED:
        _TUNED[key] = autotune_ex(sym, S, precision)
    return dict(_TUNED[key][0]), _TUNED[key][1]


def _peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text())
    return {}


class _Nvml:
    """Read-only NVML queries through the driver's libnvidia-ml (ctypes)."""

    SM = 1  # NVML_CLOCK_SM
    # Clock event reason bits of nvmlDeviceGetCurrentClocksEventReasons.
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown"}

    def __init__(self, torch_index: int):
        import ctypes

        self.C = ctypes
        lib = ctypes.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.lib = lib
        self.dev = ctypes.c_void_p()
        import torch

        uuid = str(torch.cuda.get_device_properties(torch_index).uuid)
        uuid = uuid if uuid.startswith("GPU-") else "GPU-" + uuid
        if lib.nvmlDeviceGetHandleByUUID(uuid.encode(), ctypes.byref(self.dev)) != 0:
            raise OSError("no NVML handle for " + uuid)
        self.reasons_fn = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            lib.nvmlDeviceGetCurrentClocksThrottleReasons

    def sample(self):
        C = self.C
        mhz, mx, rs = C.c_uint(), C.c_uint(), C.c_ulonglong()
        if (self.lib.nvmlDeviceGetClockInfo(self.dev, self.SM, C.byref(mhz)) or
                self.lib.nvmlDeviceGetMaxClockInfo(self.dev, self.SM, C.byref(mx)) or
                self.reasons_fn(self.dev, C.byref(rs))):
            return None
        return mhz.value, mx.value, [n for b, n in self.REASONS.items() if rs.value & b]


class ClockSampler:
    """SM clock and clock-event reasons during the timed region: NVML polled
    every millisecond from a thread, else nvidia-smi's 200 ms loop."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.out = None
        self.nvml = None
        self.samples = []
        self.thread = None
        self.stop = False
        try:
            self.nvml = _Nvml(index)
            self.nvml.sample()
        except Exception:  # noqa: BLE001  (no NVML: fall back to nvidia-smi)
            self.nvml = None

    def _poll(self):
        while not self.stop:
            smp = self.nvml.sample()
            if smp:
                self.samples.append(smp)
            time.sleep(0.001)

    def __enter__(self):
        if self.nvml:
            import threading

            self.thread = threading.Thread(target=self._poll, daemon=True)
            self.thread.start()
            return self
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.thread:
            self.stop = True
            self.thread.join(timeout=5)
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out = ""

    def summary(self) -> dict:
        if self.samples:
            sm = [x[0] for x in self.samples]
            reasons = sorted({r for x in self.samples for r in x[2]})
            return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(x[1] for x in self.samples),
                    "reasons": reasons, "samples": len(sm), "source": "nvml, 1 ms"}
        if not self.out:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm), "source": "nvidia-smi, 200 ms"}


def make_inputs(S: int, ld: int, seed0: int = 1000):
    from phdthesis_albertojimenezruiz_gb300 import Plant

    p = Plant(*DIMS)
    g = p.irradiance_batch([seed0 + s for s in range(S)], preset="c2")
    v = np.repeat(p.flat_start()[:, None], S, axis=1)
    a, b = p.companion_batch(g, v, ld=ld)
    return p, a, b


def make_conductances(p, S: int, ld: int, seed0: int = 1000) -> np.ndarray:
    """Companion conductance of every panel for the scenarios of make_inputs
    (same seeds, flat start): [n_panels, ld], columns past S zero.  With the
    plant's stamps they give the same Jacobians as make_inputs' A values."""
    g = p.irradiance_batch([seed0 + s for s in range(S)], preset="c2")
    v = np.repeat(p.flat_start()[:, None], S, axis=1)
    _, didv = p.panel_iv(p.iph(g).ravel(), v.ravel())
    out = np.zeros((p.n_panels, ld))
    out[:, :S] = -didv.reshape(p.n_panels, S)
    return out


def bytes_model(nnz_a: int, nnz_lu: int, n: int, w: int) -> dict:
    """Algorithmic bytes per scenario for each kernel (values and vectors;
    structure is shared by the batch and amortised away)."""
    return {
        "scatter": 8 * nnz_a + w * nnz_lu,
        "refactor": 2 * w * nnz_lu,
        # one pass: A's values in, the factors out (pvglu_scatter_refactor)
        "scatter_refactor": 8 * nnz_a + w * nnz_lu,
        "solve": w * nnz_lu + 4 * w * n,
        "residual": 8 * nnz_a + 8 * n + 8 * n + 4 * n,
        "update": 4 * n + 16 * n,
    }


def cpu_baseline(a: np.ndarray, b: np.ndarray, p, sym_perm, budget_s: float, threads: int,
                 prefer_ref: bool = True):
    """Reference CPU refactor+solve (level-ordered GLU + CSC solve) per scenario,
    one scenario per thread, for about `budget_s` seconds."""
    from oracle import oracle as O

    kind = "port"
    if prefer_ref and O.Ref.available():
        try:
            h = O.Ref(p.rowptr, p.colidx, sym_perm)
            kind = "reference"
        except OSError:
            h = O.Port(p.rowptr, p.colidx, sym_perm)
    else:
        h = O.Port(p.rowptr, p.colidx, sym_perm)
    S = a.shape[1]
    csc = [h.scatter(np.ascontiguousarray(a[:, s])) for s in range(min(S, threads))]
    n = p.n
    rhs = [np.random.default_rng(s).uniform(-1, 1, n) for s in range(len(csc))]

    def one(k):
        lu = h.refactor(csc[k % len(csc)])
        h.solve(lu, rhs[k % len(rhs)])

    one(0)
    t0 = time.perf_counter()
    one(0)
    single = time.perf_counter() - t0
    count = max(threads, int(budget_s * threads / max(single, 1e-6)))
    count = min(count, 200000)
    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(one, range(count)))
    dt = time.perf_counter() - t0
    return {"value": count / dt, "unit": UNIT, "cores": threads, "kind": kind,
            "sample": f"{count} refactor+solves of the 50x24x28 plant's Jacobians "
                      f"(level-ordered GLU + CSC substitution), {threads} threads, "
                      f"one scenario per thread"}


def newton_section(p, sym, stream, S: int, seed0: int, fd_check: bool = True,
                   precision: str = "fp32", fixed_tuning=None) -> dict:
    """Device Newton driver over the reference's gmin stages (tolerance
    1e-6 * n, the reference's) for S scenarios with FP32 factors + FP64
    refinement, then the adjoint dP/dG of the plant power for every panel;
    the adjoint is checked against a central difference of two more Newton
    solves (3-scenario handle, tolerance 1e-7 on the summed voltage change)."""
    import torch

    from phdthesis_albertojimenezruiz_gb300 import (FP32, FP64, SCHED_PERSISTENT, Newton,
                                                    Numeric)

    dev = torch.device("cuda", torch.cuda.current_device())
    g_to_iph = p.info["iph_stc"] / 1000.0
    prec = FP64 if precision == "fp64" else FP32

    from phdthesis_albertojimenezruiz_gb300.glu import autotune_ex

    tuned = {}

    def setup(g_cols, tol_ir=1e-12):
        count = g_cols.shape[1]
        if count not in tuned:
            if fixed_tuning:
                tuned[count] = {"max_locals": fixed_tuning[0], "wide_threshold": 0,
                                "merge_chains": 0, "schedule": fixed_tuning[1]}
            else:
                tuned[count] = _autotune(sym,count, prec)[0]
        num = Numeric(sym, count, prec, tuning=tuned[count])
        nw = Newton.for_plant(num, p)
        ld = num.ld
        iph = np.zeros((p.n_panels, ld))
        iph[:, : g_cols.shape[1]] = p.iph(g_cols)
        v0 = np.zeros((p.n_panels, ld))
        v0[:, : g_cols.shape[1]] = p.flat_start()[:, None]
        iph_d = torch.from_numpy(iph).to(dev)
        v0_d = torch.from_numpy(v0).to(dev)
        nw.set_iph(iph_d, stream=stream)
        if prec == FP32:
            nw.set_refinement(tol_ir, IR_MAX_SWEEPS)
        return num, nw, v0_d, iph_d

    g = p.irradiance_batch([seed0 + s for s in range(S)], preset="c2")
    num, nw, v0_d, _ = setup(g)
    dpdx = np.zeros((p.n, num.ld))
    dpdx[p.inv_current, :S] = -p.v_mppt
    dpdx_d = torch.from_numpy(dpdx).to(dev)
    dpdiph = torch.zeros(p.n_panels * num.ld, dtype=torch.float64, device=dev)
    tol = 1e-6 * p.n
    # warm-up solve (graph capture, first-touch)
    nw.set_voltages(v0_d, stream=stream)
    nw.run(tol, stream=stream)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e2 = torch.cuda.Event(enable_timing=True)
    nw.set_voltages(v0_d, stream=stream)
    e0.record(stream)
    nw.run(tol, check_every=8, stream=stream)
    e1.record(stream)
    nw.adjoint(dpdx_d, dpdiph, stream=stream)
    e2.record(stream)
    torch.cuda.synchronize()
    it, out, _ = nw.results()
    bodies, graph = nw.last_run()
    newton_ms = e0.elapsed_time(e1)
    lu = "FP64 LU" if prec == FP64 else "FP32 LU + FP64 refinement"
    res = {"workload": f"plant_{DIMS[0]}x{DIMS[1]}x{DIMS[2]}, {S} scenarios, {lu}, "
                       "gmin stages 100..0.05,off, tol 1e-6*n",
           "scenarios": S, "tuning": tuned[S],
           "iterations_min": int(it.min()), "iterations_max": int(it.max()),
           "converged": int((out == 0).sum()), "bodies_launched": bodies, "cuda_graph": graph,
           "newton_ms": newton_ms,
           "scenario_iterations_per_s": float(it.sum()) / (newton_ms / 1000.0),
           "adjoint_ms": e1.elapsed_time(e2),
           "adjoint_gradients_per_s": S * p.n_panels / (e1.elapsed_time(e2) / 1000.0)}
    del nw, num
    if fd_check:
        h = 1e-2
        d = np.random.default_rng(5).uniform(0.5, 1.0, p.n_panels)
        g0 = g[:, 0]
        g3 = np.stack([g0, g0 + h * d, g0 - h * d], 1)
        num3, nw3, v3_d, _ = setup(g3)
        nw3.set_voltages(v3_d, stream=stream)
        nw3.run(1e-7, stream=stream)
        x3 = torch.zeros(p.n * num3.ld, dtype=torch.float64, device=dev)
        nw3.solution(x3, stream=stream)
        d3 = torch.zeros(p.n_panels * num3.ld, dtype=torch.float64, device=dev)
        dp3 = np.zeros((p.n, num3.ld))
        dp3[p.inv_current, :3] = -p.v_mppt
        nw3.adjoint(torch.from_numpy(dp3).to(dev), d3, stream=stream)
        torch.cuda.synchronize()
        it3, out3, _ = nw3.results()
        x3 = x3.cpu().numpy().reshape(p.n, num3.ld)
        adj = d3.cpu().numpy().reshape(p.n_panels, num3.ld)[:, 0] * g_to_iph
        pw = -p.v_mppt * x3[p.inv_current, :3].sum(axis=0)
        fd = (pw[1] - pw[2]) / (2 * h)
        res["fd_check"] = {"direction": "U[0.5,1] per panel, h=1e-2 W/m^2",
                           "adjoint": float(adj @ d), "central_difference": float(fd),
                           "rel_err": float(abs(adj @ d - fd) / abs(fd)),
                           "plant_power_w": float(pw[0]),
                           "newton_iterations": [int(v) for v in it3],
                           "converged": int((out3 == 0).sum())}
    return res


def _plant_batch(dims, S: int, ld: int, seed0: int, preset: str):
    from phdthesis_albertojimenezruiz_gb300 import Plant

    p = Plant(*dims)
    g = p.irradiance_batch([seed0 + s for s in range(S)], preset=preset)
    v = np.repeat(p.flat_start()[:, None], S, axis=1)
    a, b = p.companion_batch(g, v, ld=ld)
    return p, a, b


def _time_blocks_ms(blk, step_args: tuple, step_kwargs: dict, stream, reps: int) -> float:
    """Scenario blocks timed as the headline is: each block runs its `reps`
    steps back to back on its own stream, joined after the last."""
    import torch

    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        blk.step(*step_args, stream=stream, join=False, **step_kwargs)
    blk.join(stream)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def _time_ms(fn, stream, reps: int) -> float:
    import torch

    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def config3_section(stream, steps: int) -> dict:
    """512 scenarios over three plant sizes, FP64: scatter of each size class,
    then one refactor + solve of all classes with one launch per level
    (pvglu_group), replayed from a CUDA graph; beside it the same work as one
    sequence per class."""
    import torch

    from phdthesis_albertojimenezruiz_gb300 import FP64, Numeric, Symbolic
    from phdthesis_albertojimenezruiz_gb300.glu import Group, autotune

    dims = [(10, 16, 20), (50, 24, 28), (120, 24, 28)]
    counts = [171, 171, 170]
    dev = torch.device("cuda", torch.cuda.current_device())
    members, a_d, b_d, x_d, sizes = [], [], [], [], []
    ml = None
    for k, (d, S) in reversed(list(enumerate(zip(dims, counts)))):
        ld = ((S + 63) // 64) * 64
        p, a, b = _plant_batch(d, S, ld, 7000 + 1000 * k, "c3")
        sym = Symbolic(p.rowptr, p.colidx)
        # A group launch lays out the widest table of its members: one table
        # budget for all, tuned on the largest class.
        if ml is None:
            ml = autotune(sym, S, FP64)[0]
        num = Numeric(sym, S, FP64, 0, max_locals=ml)
        members.append(num)
        a_d.append(torch.from_numpy(a).to(dev))
        b_d.append(torch.from_numpy(b).to(dev))
        x_d.append(torch.zeros_like(b_d[-1]))
        sizes.append({"plant": "x".join(map(str, d)), "unknowns": p.n, "scenarios": S,
                      "max_locals": ml})
    group = Group(members)

    def grouped():
        for num, a, b, x in zip(members, a_d, b_d, x_d):
            num.scatter(a, stream=stream)
            x.copy_(b)
        group.refactor_solve(x_d, original=True, stream=stream)

    def separate():
        for num, a, b, x in zip(members, a_d, b_d, x_d):
            num.scatter(a, stream=stream)
            x.copy_(b)
            num.refactor(stream=stream)
            num.solve(x, original=True, stream=stream)

    for _ in range(3):
        grouped()
        separate()
    ms_group = _time_ms(grouped, stream, steps)
    ms_sep = _time_ms(separate, stream, steps)
    graph = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        with torch.cuda.graph(graph, stream=side):
            for num, a, b, x in zip(members, a_d, b_d, x_d):
                num.scatter(a, stream=side)
                x.copy_(b)
            group.refactor_solve(x_d, original=True, stream=side)
    torch.cuda.synchronize()
    ms_graph = _time_ms(graph.replay, torch.cuda.current_stream(), steps)
    codes = [m.check()[0] for m in members]
    total = sum(counts)
    del group, members, a_d, b_d, x_d
    newton = config3_newton(dims, counts)
    return {"workload": "512 scenarios over plants 10x16x20, 50x24x28, 120x24x28; FP64 scatter + "
                        "refactor + solve per step", "classes": sizes,
            "value": total / (ms_graph / 1000.0), "unit": UNIT,
            "ms_per_step_graph": ms_graph, "ms_per_step_group": ms_group,
            "ms_per_step_one_sequence_per_class": ms_sep, "status_codes": codes,
            "newton": newton}


def config3_newton(dims, counts) -> dict:
    """The three-size batch as Newton loops: each size class has its own
    autotuned FP64 handle and device Newton driver (the iteration body
    captured once as a CUDA graph and replayed), seeded cloud fields of 3-8
    shadows per scenario, all three classes running at once on their own
    streams from flat starts through the gmin stages to convergence."""
    import torch

    from phdthesis_albertojimenezruiz_gb300 import FP64, Newton, Numeric, Plant, Symbolic
    from phdthesis_albertojimenezruiz_gb300.glu import autotune_ex

    dev = torch.device("cuda", torch.cuda.current_device())
    lanes = []
    for k, (d, S) in enumerate(zip(dims, counts)):
        p = Plant(*d)
        sym = Symbolic(p.rowptr, p.colidx)
        tt, _ = _autotune(sym,S, FP64)
        num = Numeric(sym, S, FP64, tuning=tt)
        nw = Newton.for_plant(num, p)
        ld = num.ld
        g = p.irradiance_batch([7000 + 1000 * k + s for s in range(S)], preset="c3")
        st = torch.cuda.Stream()
        iph = torch.from_numpy(_pad(p.iph(g), ld)).to(dev)
        v0 = torch.from_numpy(_pad(np.repeat(p.flat_start()[:, None], S, 1), ld)).to(dev)
        nw.set_iph(iph, stream=st)
        lanes.append({"plant": "x".join(map(str, d)), "p": p, "num": num, "nw": nw, "st": st,
                      "v0": v0, "tuning": tt})

    def run(lane):
        lane["nw"].set_voltages(lane["v0"], stream=lane["st"])
        lane["nw"].run(1e-6 * lane["p"].n, check_every=8, stream=lane["st"])

    for lane in lanes:  # warm-up: graph capture, first touch
        run(lane)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=len(lanes)) as ex:
        list(ex.map(run, lanes))
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    classes, iters, conv = [], 0, 0
    for lane in lanes:
        it, out, _ = lane["nw"].results()
        bodies, graph = lane["nw"].last_run()
        iters += int(it.sum())
        conv += int((out == 0).sum())
        classes.append({"plant": lane["plant"], "scenarios": int(len(it)),
                        "iterations_min": int(it.min()), "iterations_max": int(it.max()),
                        "converged": int((out == 0).sum()), "cuda_graph": graph,
                        "tuning": lane["tuning"]})
    return {"workload": "Newton to convergence (gmin stages, tol 1e-6*n) of all 512 scenarios, "
                        "three size classes on three streams at once, FP64",
            "wall_s": wall, "scenario_iterations_per_s": iters / wall,
            "refactor_solves_per_s": iters / wall, "converged": conv, "classes": classes}


def config4_section(stream, steps: int) -> dict:
    """The largest plant (200x24x28, 135k unknowns), 64 scenarios, FP32
    factors + FP64 refinement, with its error against the FP64 factors."""
    import torch

    from phdthesis_albertojimenezruiz_gb300 import FP32, FP64, Numeric, Symbolic
    from phdthesis_albertojimenezruiz_gb300.glu import autotune_ex

    S, ld = 64, 64
    p, a, b = _plant_batch((200, 24, 28), S, ld, 9000, "c4")
    sym = Symbolic(p.rowptr, p.colidx)
    dev = torch.device("cuda", torch.cuda.current_device())
    a_d = torch.from_numpy(a).to(dev)
    b_d = torch.from_numpy(b).to(dev)
    x_d = torch.zeros_like(b_d)
    t4, _ = _autotune(sym,S, FP32)
    num = Numeric(sym, S, FP32, tuning=t4)
    sweeps = torch.zeros(ld, dtype=torch.int32, device=dev)

    def step():
        num.scatter_refactor(a_d, stream=stream)
        num.solve_refined(a_d, b_d, x_d, tol=IR_TOL, max_sweeps=IR_MAX_SWEEPS, sweeps=sweeps,
                          stream=stream)

    for _ in range(3):
        step()
    ms = _time_ms(step, stream, steps)
    sw = sweeps.cpu().numpy()[:S]
    num64 = Numeric(sym, S, FP64, 0)
    num64.scatter(a_d, stream=stream)
    num64.refactor(stream=stream)
    x64 = b_d.clone()
    num64.solve(x64, original=True, stream=stream)
    torch.cuda.synchronize()
    xa, xb = x_d.cpu().numpy()[:, :S], x64.cpu().numpy()[:, :S]
    err = float(np.max(np.abs(xa - xb).max(axis=0) / np.abs(xb).max(axis=0)))
    # Every scenario against the oracle's FP64 path (sequential GLU + CSC
    # substitution on the CPU, the reference's arithmetic).
    from oracle import oracle as O

    port = O.Port(p.rowptr, p.colidx, sym.array("perm_amd"))
    errs = []
    for k in range(S):
        _, x_ref = port.scatter_refactor_solve(a[:, k], b[:, k])
        errs.append(float(np.abs(xa[:, k] - x_ref).max() / np.abs(x_ref).max()))
    return {"workload": f"plant_200x24x28 ({sym.n} unknowns, nnz_lu {int(sym.nnz_lu)}), 64 "
                        "scenarios, scatter + FP32 refactor + FP64-refined solve",
            "value": S / (ms / 1000.0), "unit": UNIT, "ms_per_step": ms,
            "tuning": t4, "sweeps_max": int(sw.max()),
            "not_converged": int((sw <= 0).sum()), "max_rel_err_vs_gpu_fp64": err,
            "per_scenario": {"sweeps": [int(v) for v in sw],
                             "rel_err_vs_oracle_fp64": [float(f"{e:.2e}") for e in errs]},
            "max_rel_err_vs_oracle_fp64": max(errs)}


def newton_iterates_section(stream, S: int, steps: int) -> dict:
    """FP32 + refinement against FP64 on Jacobians of real Newton iterates.

    The headline times companion Jacobians at the flat start.  Here the FP64
    device Newton of the 35k plant is run, for the headline's S scenarios,
    through the gmin stages up to and including stage j; the Jacobian of each
    scenario at its iterate there (with that stage's convergence conductance)
    is then solved by scatter + FP32 refactor + FP64 refinement and by
    scatter + FP64 refactor + solve, both timed, with the refinement's sweep
    counts and its error against the FP64 solution."""
    import torch

    from phdthesis_albertojimenezruiz_gb300 import (FP32, FP64, GMIN_STAGES, SCHED_LEVELS,
                                                    Newton, Numeric, Plant, Symbolic)
    from phdthesis_albertojimenezruiz_gb300.glu import autotune_ex

    p = Plant(*DIMS)
    sym = Symbolic(p.rowptr, p.colidx)
    ld = ((S + 63) // 64) * 64
    dev = torch.device("cuda", torch.cuda.current_device())
    g = p.irradiance_batch([1000 + s for s in range(S)], preset="c2")
    t64, _ = _autotune(sym,S, FP64)
    t32, _ = _autotune(sym,S, FP32)
    nt = Numeric(sym, S, FP64, tuning=t64)
    nw = Newton.for_plant(nt, p)
    nw.set_iph(torch.from_numpy(_pad(p.iph(g), ld)).to(dev))
    v0 = torch.from_numpy(_pad(np.repeat(p.flat_start()[:, None], S, 1), ld)).to(dev)
    n32 = Numeric(sym, S, FP32, tuning=t32)
    n64 = Numeric(sym, S, FP64, tuning=t64)
    sweeps = torch.zeros(ld, dtype=torch.int32, device=dev)
    out = []
    for j in (0, 2, 5, 8, 10, 11):
        nw.set_voltages(v0)
        nw.run(1e-6 * p.n, gmin=GMIN_STAGES[:j + 1])
        v = torch.as_tensor(_VoltView(nw.voltages_ptr(), p.n_panels * ld),
                            device=dev).cpu().numpy().reshape(p.n_panels, ld)[:, :S]
        gm = GMIN_STAGES[j]
        a, b = p.companion_batch(g, v, ld=ld, gmin=gm)
        a_d = torch.from_numpy(a).to(dev)
        b_d = torch.from_numpy(b).to(dev)
        x32 = torch.zeros_like(b_d)
        x64 = torch.empty_like(b_d)

        def step32():
            n32.scatter_refactor(a_d, stream=stream)
            n32.solve_refined(a_d, b_d, x32, tol=IR_TOL, max_sweeps=40, sweeps=sweeps,
                              stream=stream)

        def step64():
            if t64["schedule"] == SCHED_LEVELS:  # scatter + refactor in one pass
                n64.scatter_refactor(a_d, stream=stream)
                x64.copy_(b_d)
                n64.solve(x64, original=True, stream=stream)
            else:  # refactor + solve in one persistent launch
                n64.scatter(a_d, stream=stream)
                x64.copy_(b_d)
                n64.refactor_solve(x64, original=True, stream=stream)

        for _ in range(3):
            step32()
            step64()
        ms32 = _time_ms(step32, stream, steps)
        ms64 = _time_ms(step64, stream, steps)
        sw = sweeps.cpu().numpy()[:S]
        xa, xb = x32.cpu().numpy()[:, :S], x64.cpu().numpy()[:, :S]
        err = np.abs(xa - xb).max(axis=0) / np.abs(xb).max(axis=0)
        out.append({"stage": j, "gmin": gm if gm > 0 else None,
                    "fp32ir_per_s": S / (ms32 / 1000.0), "fp64_per_s": S / (ms64 / 1000.0),
                    "fp32ir_over_fp64": ms64 / ms32,
                    "sweeps_histogram": {str(int(k)): int((sw == k).sum()) for k in np.unique(sw)},
                    "not_converged": int((sw <= 0).sum()),
                    "max_rel_err_vs_fp64": float(err[sw > 0].max()) if (sw > 0).any() else None})
        del a_d, b_d, x32, x64
    return {"workload": f"plant_50x24x28, {S} scenarios, Jacobians at the FP64 Newton iterate "
                        "at the end of gmin stage j (stage j's conductance included); "
                        "refinement tolerance 1e-12, up to 40 sweeps", "stages": out}


def wide_section(stream, steps: int, S: int = 512, patterns: str = "ref,mesh,random",
                 profile: bool = False, profile_max_locals: int = 24) -> dict:
    """Patterns whose factors have columns and rows too wide for a chain-
    program table (run as WIDE program levels, a block per unit): the
    reference's own plant topology with the reference's AMD ordering (7
    blocks x 50 strings x 50 panels, 34,717 unknowns, bus columns and rows of
    2,455 entries, 100 U levels), and two fill-heavy test patterns.  Per
    pattern: the single-instance FP64 path in each schedule, the batched FP64
    path (S scenarios, HBM fraction of scatter + refactor + solve), the
    batched FP32 + refinement path, and the reference's CPU path (the
    oracle's sequential GLU + substitution, one core) on the same matrix."""
    import torch

    sys.path.insert(0, str(ROOT / "tests"))
    import matrices as M
    from oracle import oracle as O
    from phdthesis_albertojimenezruiz_gb300 import (FP32, FP64, SCHED_LEVELS, SCHED_PERSISTENT,
                                                    SCHED_THREAD_CHAIN, Blocks, Numeric,
                                                    Symbolic)
    from phdthesis_albertojimenezruiz_gb300.glu import autotune_ex
    from phdthesis_albertojimenezruiz_gb300.plant import block_plant

    dev = torch.device("cuda", torch.cuda.current_device())
    peak = _peaks().get("hbm_gbs")
    with np.load(ROOT / "tests" / "golden" / "orderings" / "block_plant_amd.npz") as z:
        perm7 = z["perm_7x50x50"]
    cases = []
    wanted = {p.strip() for p in patterns.split(",")}
    if "ref" in wanted:
        cols = [block_plant(7, 50, 50, seed=300 + k) for k in range(8)]
        cases.append(("reference_topology_7x50x50 (reference AMD ordering)", cols[0][0],
                      cols[0][1], perm7, np.stack([c[2] for c in cols], 1),
                      np.stack([c[3] for c in cols], 1)))
    for key, name in (("mesh", "mesh_30x30"), ("random", "random_1500")):
        if key in wanted:
            rp, ci, a, b = M.CASES[name]()
            cases.append((name, rp, ci, None, a[:, None], b[:, None]))
    out = []
    for name, rp, ci, perm, a_few, b_few in cases:
        sym = Symbolic(rp, ci, perm)
        n, nnz_a, nnz_lu = sym.n, int(sym.nnz_a), int(sym.nnz_lu)
        res = {"pattern": name, "n": n, "nnz_a": nnz_a, "nnz_lu": nnz_lu,
               "lu_levels": sym.info["lu_levels"], "u_levels": sym.info["u_levels"]}
        # Single instance, FP64, every schedule (not in profiling runs, which
        # time the batched FP64 step alone with the autotuner's choice for
        # the reference topology fixed).
        a1 = torch.from_numpy(np.ascontiguousarray(a_few[:, 0])).to(dev)
        b1 = torch.from_numpy(np.ascontiguousarray(b_few[:, 0])).to(dev)
        x1 = b1.clone()
        single = {}
        for sname, sched in (() if profile else (("thread_chain_levels", SCHED_THREAD_CHAIN),
                                                  ("programs_levels", SCHED_LEVELS),
                                                  ("programs_persistent", SCHED_PERSISTENT),
                                                  ("programs_autotuned", None))):
            if sched is None:
                t1, _ = _autotune(sym, 1, FP64)
                one = Numeric(sym, 1, FP64, tuning=t1)
                res["single_autotuned"] = {"tuning": t1, "program_info": one.info}
            else:
                one = Numeric(sym, 1, FP64, sched)

            def plain_step():
                one.scatter(a1, stream=stream)
                x1.copy_(b1)
                one.refactor_solve(x1, original=True, stream=stream)

            for _ in range(3):
                plain_step()
            single[sname] = 1000.0 / _time_ms(plain_step, stream, max(10, steps))
            if sched == SCHED_LEVELS:
                res["single_program_info"] = one.info
            del one
        res["single_fp64_per_s"] = single
        # Batched: S scenarios (the distinct Jacobians tiled).
        ld = ((S + 63) // 64) * 64
        reps = -(-S // a_few.shape[1])
        a = np.zeros((nnz_a, ld))
        b = np.zeros((n, ld))
        a[:, :S] = np.tile(a_few, (1, reps))[:, :S]
        b[:, :S] = np.tile(b_few, (1, reps))[:, :S]
        a_d = torch.from_numpy(a).to(dev)
        b_d = torch.from_numpy(b).to(dev)
        if profile:
            t64 = {"max_locals": profile_max_locals, "wide_threshold": 0, "merge_chains": 2,
                   "schedule": SCHED_LEVELS}
        else:
            t64, _ = _autotune(sym, S, FP64)
        n64 = Numeric(sym, S, FP64, tuning=t64)
        x64 = torch.empty_like(b_d)

        def step64():
            n64.scatter(a_d, stream=stream)
            x64.copy_(b_d)
            n64.refactor_solve(x64, original=True, stream=stream)

        for _ in range(3):
            step64()
        ms64 = _time_ms(step64, stream, steps)
        bm = bytes_model(nnz_a, nnz_lu, n, 8)
        byt = (bm["scatter"] + bm["refactor"] + bm["solve"]) * S
        res["batched_fp64"] = {
            "value": S / (ms64 / 1000.0), "unit": UNIT, "ms_per_step": ms64,
            "tuning": t64, "program_info": n64.info,
            "hbm": {"bytes_per_step": byt, "achieved_gbs": byt / (ms64 / 1000.0) / 1e9,
                    "frac": byt / (ms64 / 1000.0) / 1e9 / peak if peak else None}}
        if not profile and S % 4 == 0 and S // 4 >= 128 and t64["schedule"] == SCHED_LEVELS:
            # The same step as 4 scenario blocks of at least 128 scenarios
            # (smaller blocks leave the long chains' lanes half empty: 2
            # blocks of 32 took 1.79 ms against 1.14 ms for one handle of 64).
            Hb = S // 4
            blk = Blocks(sym, S, 4, FP64, tuning=t64)

            def block_cols(t, k, ld_k):
                out_ = torch.zeros((t.shape[0], ld_k), dtype=t.dtype, device=dev)
                out_[:, :Hb] = t[:, k * Hb:(k + 1) * Hb]
                return out_

            ak = [block_cols(a_d, k, blk.parts[k].ld) for k in range(4)]
            bk = [block_cols(b_d, k, blk.parts[k].ld) for k in range(4)]
            xk = [torch.empty_like(t) for t in bk]

            def step_blocks():
                blk.step(ak, bk, xk, stream=stream)

            for _ in range(3):
                step_blocks()
            msb = _time_blocks_ms(blk, (ak, bk, xk), {}, stream, steps)
            res["batched_fp64"]["blocks"] = {
                "value": S / (msb / 1000.0), "unit": UNIT, "ms_per_step": msb, "blocks": 4,
                "bit_identical_to_one_handle": bool(all(
                    torch.equal(xk[k][:, :Hb], x64[:, k * Hb:(k + 1) * Hb]) for k in range(4)))}
            del blk, ak, bk, xk
        if profile:
            out.append(res)
            del n64, a_d, b_d, x64
            continue
        t32, _ = _autotune(sym, S, FP32)
        n32 = Numeric(sym, S, FP32, tuning=t32)
        x32 = torch.zeros_like(b_d)
        sweeps = torch.zeros(ld, dtype=torch.int32, device=dev)

        def step32():
            n32.scatter(a_d, stream=stream)
            n32.refactor(stream=stream)
            n32.solve_refined(a_d, b_d, x32, tol=IR_TOL, max_sweeps=30, sweeps=sweeps,
                              stream=stream)

        for _ in range(3):
            step32()
        ms32 = _time_ms(step32, stream, steps)
        sw = sweeps.cpu().numpy()[:S]
        xa, xb = x32.cpu().numpy()[:, :S], x64.cpu().numpy()[:, :S]
        res["batched_fp32ir"] = {
            "value": S / (ms32 / 1000.0), "unit": UNIT, "ms_per_step": ms32,
            "tuning": t32,
            "sweeps_max": int(sw.max()), "not_converged": int((sw <= 0).sum()),
            "max_rel_err_vs_fp64": float(np.max(np.abs(xa - xb).max(axis=0) /
                                                np.abs(xb).max(axis=0)))}
        # The oracle (the reference's sequential arithmetic) on scenario 0,
        # timed on one core, and checked against the batched FP64 factors.
        port = O.Port(rp, ci, sym.array("perm_amd"))
        t0 = time.perf_counter()
        cnt = 0
        while cnt < 3 or time.perf_counter() - t0 < 1.0:
            lu_ref, x_ref = port.scatter_refactor_solve(a[:, 0], b[:, 0])
            cnt += 1
        res["cpu_oracle_1core_per_s"] = cnt / (time.perf_counter() - t0)
        res["batched_fp64_bit_identical_to_oracle"] = bool(np.array_equal(xb[:, 0], x_ref))
        out.append(res)
        del n64, n32, a_d, b_d, x64, x32
    return {"workload": f"WIDE program levels: single instance and {S} scenarios per step, "
                        "scatter + refactor + solve", "patterns": out}


def _newton_handle(p, sym, S: int, precision, tol_ir: float = 1e-12):
    from phdthesis_albertojimenezruiz_gb300 import FP32, Newton, Numeric
    from phdthesis_albertojimenezruiz_gb300.glu import autotune_ex

    t, _ = _autotune(sym,S, precision)
    num = Numeric(sym, S, precision, tuning=t)
    nw = Newton.for_plant(num, p)
    if precision == FP32:
        nw.set_refinement(tol_ir, IR_MAX_SWEEPS)
    return num, nw


def _pad(a: np.ndarray, ld: int) -> np.ndarray:
    out = np.zeros((a.shape[0], ld))
    out[:, : a.shape[1]] = a
    return out


def config1_section() -> dict:
    """4x8x20 plant (652 unknowns), FP64 Newton on the device to a Kirchhoff
    mismatch below 1e-9 A, against the CPU oracle's Newton loop on the same
    input (bit-identical expected) with both timed."""
    import torch

    from oracle import oracle as O
    from phdthesis_albertojimenezruiz_gb300 import FP64, GMIN_STAGES, Plant, Symbolic

    p = Plant(4, 8, 20)
    sym = Symbolic(p.rowptr, p.colidx)
    g = p.irradiance(seed=1, preset="c1")
    num, nw = _newton_handle(p, sym, 1, FP64)
    tol = 1e-9
    iph = p.iph(g)
    nw.set_iph(torch.from_numpy(iph).cuda())
    nw.set_voltages(torch.from_numpy(p.flat_start()).cuda())
    nw.run(tol)  # warm-up (graph capture)
    torch.cuda.synchronize()
    nw.set_voltages(torch.from_numpy(p.flat_start()).cuda())
    t0 = time.perf_counter()
    nw.run(tol)
    gpu_s = time.perf_counter() - t0
    it, out, _ = nw.results()
    x = torch.zeros(p.n, dtype=torch.float64, device="cuda")
    nw.solution(x)
    mm = float(nw.mismatch()[0])
    port = O.Port(p.rowptr, p.colidx, sym.array("perm_amd"))
    t0 = time.perf_counter()
    rc, it_o, _, _, x_o = port.newton(p, iph, p.flat_start(), GMIN_STAGES, tol)
    cpu_s = time.perf_counter() - t0
    return {"workload": f"plant_4x8x20 ({p.n} unknowns), FP64 Newton, gmin stages, "
                        f"tol {tol} on sum |dV|", "iterations": int(it[0]),
            "oracle_iterations": it_o, "converged": bool(out[0] == 0 and rc == 0),
            "kcl_mismatch_a": mm, "bit_identical_to_oracle": bool(np.array_equal(x.cpu().numpy(), x_o)),
            "gpu_newton_s": gpu_s, "cpu_oracle_newton_s": cpu_s}


def config2_section() -> dict:
    """The 35k plant over 300 time steps (t = 0..299 s, 5 shadows drifting at
    5-15 m/s): the photocurrents of every step come from the device
    irradiance field and all steps are solved as one batch, FP64."""
    import torch

    from phdthesis_albertojimenezruiz_gb300 import FP64, Plant, Symbolic

    p = Plant(*DIMS)
    sym = Symbolic(p.rowptr, p.colidx)
    T = 300
    num, nw = _newton_handle(p, sym, T, FP64)
    ld = num.ld
    sh = p.shadows(2024, "c2")
    # scenario t sees the field at time t (dt = 1 s); photocurrents straight
    # into the driver from the device field
    nw.set_field(p.pan_x, p.pan_y, [sh] * T, iph_per_g=p.info["iph_stc"] / 1000.0,
                 t_offset=np.arange(T, dtype=np.float64))
    nw.field_iph(0.0)
    v0 = torch.from_numpy(_pad(np.repeat(p.flat_start()[:, None], T, 1), ld)).cuda()
    tol = 1e-6 * p.n
    nw.set_voltages(v0)
    nw.run(tol)
    torch.cuda.synchronize()
    nw.set_voltages(v0)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    nw.run(tol)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    it, out, _ = nw.results()
    del nw, num
    seq = config2_sequential(p, sym, sh, T)
    return {"workload": "plant_50x24x28, 300 time steps of one 5-shadow field as one FP64 "
                        "batch, gmin stages, tol 1e-6*n", "time_steps": T,
            "newton_ms": ms, "time_steps_per_s": T / (ms / 1000.0),
            "iterations_min": int(it.min()), "iterations_max": int(it.max()),
            "converged": int((out == 0).sum()),
            "refactor_solves_per_s": float(it.sum()) / (ms / 1000.0),
            "single_instance_sequential": seq,
            "batch_over_sequential": seq["wall_s"] * 1000.0 / ms}


def config2_sequential(p, sym, shadows, T: int) -> dict:
    """The plain single-instance FP64 path over the same 300 snapshots, in
    sequence, as the reference's simulator runs them
    (000_PVPP_simulator.cpp:120-236: each snapshot from the flat start
    through the gmin stages): one scenario handle with the fastest
    single-instance schedule, the snapshot's photocurrents from the device
    field at t, the Newton body replayed from its CUDA graph."""
    import torch

    num, nw = _newton_handle(p, sym, 1, 0)
    nw.set_field(p.pan_x, p.pan_y, [shadows], iph_per_g=p.info["iph_stc"] / 1000.0)
    v0 = torch.from_numpy(p.flat_start()).cuda()
    tol = 1e-6 * p.n
    nw.field_iph(0.0)
    nw.set_voltages(v0)
    nw.run(tol)  # warm-up: graph capture
    torch.cuda.synchronize()
    iters, conv = [], 0
    t0 = time.perf_counter()
    for t in range(T):
        nw.field_iph(float(t))
        nw.set_voltages(v0)
        nw.run(tol, check_every=16)
        it, out, _ = nw.results()
        iters.append(int(it[0]))
        conv += int(out[0] == 0)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    return {"time_steps": T, "wall_s": wall, "time_steps_per_s": T / wall,
            "iterations_min": min(iters), "iterations_max": max(iters), "converged": conv,
            "refactor_solves_per_s": sum(iters) / wall}


def config5_fd_section(precision_name: str) -> dict:
    """Per-panel dP/dG of the 35k plant, the 128-scenario batch of the
    differentiation configuration, checked on scenario 0:
    * against central differences at h = 1e-3 W/m^2 on 200 random panels,
      each difference solved in extended precision by the oracle on the
      panel's inverter block (the plant decomposes by inverter, so the plant
      power moves only through that inverter's power);
    * against the oracle's CPU FP64 adjoint (the reference's factors) on
      every panel.
    Beside them, the same differences taken from the GPU's own FP64 Newton
    solves on 20 of those panels (40 extra scenarios in the batch), which
    shows the FP64 floor of such differences."""
    import torch

    from oracle import oracle as O
    from phdthesis_albertojimenezruiz_gb300 import FP32, FP64, Plant, Symbolic

    prec = FP64 if precision_name == "fp64" else FP32
    p = Plant(*DIMS)
    sym = Symbolic(p.rowptr, p.colidx)
    g_to_iph = p.info["iph_stc"] / 1000.0
    rng = np.random.default_rng(77)
    panels = rng.choice(p.n_panels, 200, replace=False)
    h = 1e-3
    base = [p.irradiance(seed=5000 + s, preset="c2") for s in range(128)]
    g0 = base[0]
    cols = list(base)
    gpu_fd_panels = panels[:20]
    for k in gpu_fd_panels:
        for sign in (1.0, -1.0):
            gk = g0.copy()
            gk[k] += sign * h
            cols.append(gk)
    G = np.stack(cols, 1)
    S = G.shape[1]
    num, nw = _newton_handle(p, sym, S, prec)
    ld = num.ld
    nw.set_iph(torch.from_numpy(_pad(p.iph(G), ld)).cuda())
    nw.set_voltages(torch.from_numpy(_pad(np.repeat(p.flat_start()[:, None], S, 1), ld)).cuda())
    nw.run(1e-7)
    x = torch.zeros(p.n * ld, dtype=torch.float64, device="cuda")
    nw.solution(x)
    dpdx = np.zeros((p.n, ld))
    dpdx[p.inv_current, :S] = -p.v_mppt
    grad = torch.zeros(p.n_panels * ld, dtype=torch.float64, device="cuda")
    nw.adjoint(torch.from_numpy(dpdx).cuda(), grad)
    torch.cuda.synchronize()
    it, out, _ = nw.results()
    x = x.cpu().numpy().reshape(p.n, ld)
    v = torch.as_tensor(_VoltView(nw.voltages_ptr(), p.n_panels * ld),
                        device="cuda").cpu().numpy().reshape(p.n_panels, ld)[:, 0]
    full = grad.cpu().numpy().reshape(p.n_panels, ld)[:, 0] * g_to_iph
    adj = full[panels]
    # Extended-precision central differences on the inverter blocks.
    per_inv = DIMS[1] * DIMS[2]
    q = Plant(1, DIMS[1], DIMS[2])
    qs = Symbolic(q.rowptr, q.colidx)
    qport = O.Port(q.rowptr, q.colidx, qs.array("perm_amd"))
    qdpdx = np.zeros(q.n)
    qdpdx[q.inv_current] = -q.v_mppt
    iph0 = p.iph(g0)

    def ext(k):
        _, pans = p.inverter_block(int(k) // per_inv)
        fd, _, res = qport.fd_ext(q, iph0[pans], v[pans], qdpdx, int(k) - pans.start,
                                  g_to_iph * h)
        return g_to_iph * fd, res

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
        ext_out = list(ex.map(ext, panels))
    ext_s = time.perf_counter() - t0
    fd = np.array([e[0] for e in ext_out])
    rel = np.abs(adj - fd) / np.abs(fd)
    # The GPU's own FP64 differences, inverter power by inverter power.
    xs = x[:, 128:S]
    gpu_rel = []
    for j, k in enumerate(gpu_fd_panels):
        inv = int(k) // per_inv
        pw = -p.v_mppt * xs[p.inv_current[inv], 2 * j:2 * j + 2]
        fdk = (pw[0] - pw[1]) / (2 * h)
        gpu_rel.append(abs(full[k] - fdk) / abs(fdk))
    # The FP64 CPU adjoint of the oracle (factors bit-identical to the
    # reference's) at the same operating point, every panel.
    port = O.Port(p.rowptr, p.colidx, sym.array("perm_amd"))
    dpdx1 = np.zeros(p.n)
    dpdx1[p.inv_current] = -p.v_mppt
    ref = port.adjoint(p, p.iph(g0), v, dpdx1) * g_to_iph
    return {"workload": f"plant_50x24x28, 128 scenarios, {precision_name} forward; dP/dG of "
                        "scenario 0 on 200 random panels against central differences "
                        f"(h = {h} W/m^2)", "scenarios": S,
            "converged": int((out == 0).sum()),
            "fd_max_rel_err": float(rel.max()), "fd_median_rel_err": float(np.median(rel)),
            "fd_max_abs_err_over_max_grad": float(np.abs(adj - fd).max() / np.abs(adj).max()),
            "fd_method": "each +-h pair solved in long double (Newton in correction form, "
                         "residual in long double, FP64 Jacobian) on the panel's inverter block "
                         "by the oracle, from the GPU's converged voltages",
            "fd_seconds": ext_s,
            "gpu_fp64_fd_20_panels": {
                "max_rel_err": float(max(gpu_rel)), "median_rel_err": float(np.median(gpu_rel)),
                "note": "differences of the GPU's FP64 Newton solves (inverter power): node "
                        "voltages near 1 kV are quantised at 2.3e-13 V, about 1e-8 W of "
                        "inverter power, against 1e-5 to 1e-2 W of difference"},
            "vs_cpu_fp64_adjoint_all_panels_max_rel": float(
                np.abs(full - ref).max() / np.abs(ref).max()),
            "max_grad_w_per_w_m2": float(np.abs(full).max())}


class _VoltView:
    def __init__(self, ptr, count):
        self.__cuda_array_interface__ = {"shape": (count,), "typestr": "<f8",
                                         "data": (ptr, False), "version": 3}


def run_configs(args, stream) -> dict:
    wanted = {c.strip() for c in args.configs.split(",") if c.strip()}
    out = {}
    seconds = {}
    sections = [
        ("1", "config1", lambda: config1_section()),
        ("2", "config2", lambda: config2_section()),
        ("3", "config3", lambda: config3_section(stream, max(5, args.steps))),
        ("4", "config4", lambda: config4_section(stream, max(5, args.steps))),
        ("5", "config5_fd", lambda: {m: config5_fd_section(m) for m in ("fp64", "fp32")}),
        ("i", "fp32ir_on_newton_iterates",
         lambda: newton_iterates_section(stream, args.scenarios, max(5, args.steps))),
        ("w", "wide_units",
         lambda: wide_section(stream, max(5, args.steps), args.scenarios, args.wide_patterns,
                              args.wide_profile, args.wide_max_locals)),
    ]
    for tag, key, fn in sections:
        if tag in wanted:
            t0 = time.perf_counter()
            out[key] = fn()
            seconds[key] = round(time.perf_counter() - t0, 1)
    if seconds:
        out["section_seconds"] = seconds
    return out


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from phdthesis_albertojimenezruiz_gb300 import Symbolic

    threads = os.cpu_count() or 1
    S = threads
    p, a, b = make_inputs(S, S)
    sym = Symbolic(p.rowptr, p.colidx)
    perm = sym.array("perm_amd")
    res = None
    for _ in range(args.warmup):
        cpu_baseline(a, b, p, perm, 1.0, threads)
    vals, walls = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        res = cpu_baseline(a, b, p, perm, 3.0, threads)
        walls.append(time.perf_counter() - t0)
        vals.append(res["value"])
    value = float(np.median(vals))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        # A step is one bounded sample (about 3 s of refactor+solves on all
        # host threads), so its wall time is reported as the step time.
        "ms_per_step": 1000.0 * float(np.median(walls)), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "plant_50x24x28 (33,750 unknowns) refactor+solve, CPU GLU",
                   "scenarios_per_step": threads},
        "cpu_baseline": dict(res, value=value),
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main() -> None:
    global IR_TOL, IR_MAX_SWEEPS
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--scenarios", type=int, default=512)
    ap.add_argument("--cpu-budget", type=float, default=10.0)
    ap.add_argument("--ir-tol", type=float, default=IR_TOL,
                    help="refinement stop: max|dx| <= tol * max|x| per scenario")
    ap.add_argument("--ir-sweeps", type=int, default=IR_MAX_SWEEPS)
    ap.add_argument("--only-batched", action="store_true",
                    help="time the batched FP32+IR path only (profiling runs)")
    ap.add_argument("--blocks", type=int, default=HEADLINE_BLOCKS,
                    help="scenario blocks of the headline step, each on its own stream "
                         "(pvglu_blocks; 1: one handle)")
    ap.add_argument("--newton-scenarios", type=int, default=128,
                    help="scenarios of the device Newton + adjoint section (0: skip)")
    ap.add_argument("--only-newton", action="store_true",
                    help="run the Newton + adjoint section alone (profiling runs)")
    ap.add_argument("--newton-precision", default="fp64", choices=["fp64", "fp32"],
                    help="factor precision of the Newton section")
    ap.add_argument("--max-locals", type=int, default=0,
                    help="chain-program table size of the batched handle (0: autotune)")
    ap.add_argument("--schedule", default="persistent", choices=["levels", "persistent"],
                    help="schedule used with --max-locals (autotuned otherwise)")
    ap.add_argument("--configs", default="1,2,3,4,5,i,w",
                    help="extra workloads reported beside the headline (1: 4x8x20 Newton vs the "
                         "oracle, 2: 300 time steps, 3: three plant sizes per level launch, "
                         "4: the 135k plant, 5: per-panel adjoint vs central differences, "
                         "i: FP32 + refinement vs FP64 on Newton-iterate Jacobians, "
                         "w: wide units on the reference's plant topology and fill-heavy "
                         "patterns; empty: none)")
    ap.add_argument("--wide-patterns", default="ref",
                    help="patterns of the wide-unit section (ref: the reference's plant topology, "
                         "mesh: mesh_30x30, random: random_1500)")
    ap.add_argument("--wide-profile", action="store_true",
                    help="wide-unit section: the batched FP64 step alone, fixed tuning "
                         "(profiling runs)")
    ap.add_argument("--wide-max-locals", type=int, default=24,
                    help="table size of the fixed tuning of --wide-profile")
    ap.add_argument("--only-configs", action="store_true",
                    help="run the --configs workloads alone (profiling runs)")
    ap.add_argument("--newton-max-locals", type=int, default=0,
                    help="table size of the Newton handles, with --schedule (0: autotune)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    IR_TOL, IR_MAX_SWEEPS = args.ir_tol, args.ir_sweeps
    if args.impl == "reference":
        run_reference(args)
        return

    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist  # noqa: F811

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from phdthesis_albertojimenezruiz_gb300 import (FP32, FP64, SCHED_LEVELS, SCHED_PERSISTENT,
                                                    SCHED_THREAD_CHAIN, Blocks, Numeric,
                                                    Symbolic)
    from phdthesis_albertojimenezruiz_gb300.replicas import max_over_ranks

    if args.only_configs:
        out = run_configs(args, torch.cuda.current_stream())
        if rank == 0:
            print(json.dumps(out))
        return
    if args.only_newton:
        from phdthesis_albertojimenezruiz_gb300 import Plant

        p = Plant(*DIMS)
        sym = Symbolic(p.rowptr, p.colidx)
        fixed = None
        if args.newton_max_locals > 0:
            fixed = (args.newton_max_locals, SCHED_LEVELS if args.schedule == "levels"
                     else SCHED_PERSISTENT)
        res = newton_section(p, sym, torch.cuda.current_stream(), args.newton_scenarios, 5000,
                             fd_check=False, precision=args.newton_precision,
                             fixed_tuning=fixed)
        if rank == 0:
            print(json.dumps(res))
        return
    S = args.scenarios
    ld = ((S + 63) // 64) * 64
    p, a, b = make_inputs(S, ld, seed0=1000 + rank * S)
    sym = Symbolic(p.rowptr, p.colidx)
    n, nnz_a, nnz_lu = sym.n, int(sym.nnz_a), int(sym.nnz_lu)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream()
    a_d = torch.from_numpy(a).to(dev)
    b_d = torch.from_numpy(b).to(dev)
    x_d = torch.zeros_like(b_d)
    sweeps = torch.zeros(ld, dtype=torch.int32, device=dev)
    from phdthesis_albertojimenezruiz_gb300.glu import autotune

    if args.max_locals > 0:
        tuned = {"max_locals": args.max_locals,
                 "schedule": SCHED_LEVELS if args.schedule == "levels" else SCHED_PERSISTENT,
                 "source": "flags"}
    else:
        from phdthesis_albertojimenezruiz_gb300.glu import autotune_ex

        tt, tms = _autotune(sym,S, FP32)
        tuned = dict(tt, ms_scatter_refactor_solve=tms, source="pvglu_autotune_ex")
    tuning = {k: tuned.get(k, d) for k, d in (("max_locals", 0), ("wide_threshold", 0),
                                              ("merge_chains", 0), ("schedule", SCHED_LEVELS))}
    num = Numeric(sym, S, FP32, tuned["schedule"], max_locals=tuned["max_locals"],
                  tuning=tuning)
    persistent = tuned["schedule"] == SCHED_PERSISTENT
    assert num.ld == ld
    # The headline's scenario blocks: block k holds scenarios [k H, (k+1) H)
    # in buffers of its own layout (inputs resident before the timed region).
    n_blk = args.blocks if args.blocks > 1 and S % args.blocks == 0 else 1
    blk = blk_a = blk_b = blk_x = blk_sw = None
    if n_blk > 1:
        H = S // n_blk
        blk = Blocks(sym, S, n_blk, FP32, tuning=tuning)

        def block_cols(t, k, ld_k):
            out = torch.zeros((t.shape[0], ld_k), dtype=t.dtype, device=dev)
            out[:, :H] = t[:, k * H:(k + 1) * H]
            return out

        blk_a = [block_cols(a_d, k, blk.parts[k].ld) for k in range(n_blk)]
        blk_b = [block_cols(b_d, k, blk.parts[k].ld) for k in range(n_blk)]
        blk_x = [torch.zeros_like(t) for t in blk_b]
        blk_sw = [torch.zeros(blk.parts[k].ld, dtype=torch.int32, device=dev)
                  for k in range(n_blk)]

    def block_step():
        blk.step(blk_a, blk_b, blk_x, tol=IR_TOL, max_sweeps=IR_MAX_SWEEPS, sweeps=blk_sw,
                 stream=stream)

    def step():
        num.scatter_refactor(a_d, stream=stream)
        num.solve_refined(a_d, b_d, x_d, tol=IR_TOL, max_sweeps=IR_MAX_SWEEPS, sweeps=sweeps,
                          stream=stream)

    for _ in range(args.warmup):
        step()
        if blk is not None:
            block_step()
    torch.cuda.synchronize()
    for h_ in [num] + (blk.parts if blk is not None else []):
        code, col, sc = h_.check()
        if code:
            raise SystemExit(f"refactor failed: status {code} column {col} scenario {sc}")

    # Timed regions: K steps each, barrier + synchronize on both sides, CUDA
    # events on the launching stream.  The one handle first, with per-step
    # events around the one-pass scatter + refactorization (the roofline);
    # then the headline, the scenario blocks (the same 512 scenarios).
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    rf = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for k in range(args.steps):
            rf[k][0].record(stream)
            num.scatter_refactor(a_d, stream=stream)
            rf[k][1].record(stream)
            num.solve_refined(a_d, b_d, x_d, tol=IR_TOL, max_sweeps=IR_MAX_SWEEPS,
                              sweeps=sweeps, stream=stream)
        ev1.record(stream)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        ms_one = max_over_ranks(ev0.elapsed_time(ev1), dist, dev)
        ms = ms_one
        if blk is not None:
            eb0 = torch.cuda.Event(enable_timing=True)
            eb1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            eb0.record(stream)
            # Blocks are independent: each block's stream runs its K steps
            # back to back, and the timed region ends when every block has
            # finished all of them.
            for k in range(args.steps):
                blk.step(blk_a, blk_b, blk_x, tol=IR_TOL, max_sweeps=IR_MAX_SWEEPS,
                         sweeps=blk_sw, stream=stream, join=False)
            blk.join(stream)
            eb1.record(stream)
            torch.cuda.synchronize()
            if dist:
                dist.barrier()
            ms = max_over_ranks(eb0.elapsed_time(eb1), dist, dev)
    refactor_ms = float(np.mean([s.elapsed_time(e) for s, e in rf]))
    single_handle = {"value": S * world * args.steps / (ms_one / 1000.0), "unit": UNIT,
                     "ms_per_step": ms_one / args.steps,
                     "call": "one handle of all scenarios: pvglu_scatter_refactor + "
                             "pvglu_solve_refined"}
    if blk is not None:
        # The blocks' solutions and sweeps against the one handle's.
        same = all(
            torch.equal(blk_x[k][:, :S // n_blk], x_d[:, k * (S // n_blk):(k + 1) * (S // n_blk)])
            and torch.equal(blk_sw[k][:S // n_blk],
                            sweeps[k * (S // n_blk):(k + 1) * (S // n_blk)])
            for k in range(n_blk))
        single_handle["blocks_bit_identical"] = bool(same)
    # The residual kernel alone (the largest share of a step: two launches per
    # step), timed with CUDA events on the launching stream over 20 calls.
    r_buf = torch.empty(n * ld, dtype=torch.float32, device=dev)
    for _ in range(3):
        num.refine_residual(a_d, b_d, x_d, r_buf, stream=stream)
    er0 = torch.cuda.Event(enable_timing=True)
    er1 = torch.cuda.Event(enable_timing=True)
    er0.record(stream)
    for _ in range(20):
        num.refine_residual(a_d, b_d, x_d, r_buf, stream=stream)
    er1.record(stream)
    torch.cuda.synchronize()
    resid_ms = er0.elapsed_time(er1) / 20
    del r_buf
    sw = sweeps.cpu().numpy()[:S]
    value = S * world * args.steps / (ms / 1000.0)
    if args.only_batched:  # profiling runs: the batched path alone
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT,
                              "ms_per_step": ms / args.steps, "refactor_ms": refactor_ms,
                              "scenarios": S, "blocks": n_blk, "sweeps_max": int(sw.max()),
                              "single_handle": single_handle, "tuning": tuned}))
        if dist:
            dist.destroy_process_group()
        return

    # Accuracy of the refined solutions against the FP64 GPU factors.
    num64 = Numeric(sym, S, FP64, SCHED_PERSISTENT)
    num64.scatter(a_d, stream=stream)
    num64.refactor(stream=stream)
    x64 = b_d.clone()
    num64.solve(x64, original=True, stream=stream)
    torch.cuda.synchronize()
    xa = x_d.cpu().numpy()[:, :S]
    xb = x64.cpu().numpy()[:, :S]
    max_rel = float(np.max(np.abs(xa - xb).max(axis=0) / np.abs(xb).max(axis=0)))
    del num64
    # And against the oracle's FP64 path (the reference's sequential GLU and
    # substitution on the CPU) for a sample of scenarios.
    from oracle import oracle as O

    port = O.Port(p.rowptr, p.colidx, sym.array("perm_amd"))
    oracle_err = []
    for k in sorted({0, 1, S // 3, S // 2, (2 * S) // 3, S - 1}):
        _, x_ref = port.scatter_refactor_solve(a[:, k], b[:, k])
        oracle_err.append(float(np.abs(xa[:, k] - x_ref).max() / np.abs(x_ref).max()))

    # The same step with the refinement stopped at the benchmark spec's accuracy
    # bar (1e-10 relative to the FP64 oracle) instead of 1e-12: its rate,
    # sweeps and errors, reported beside the headline (which keeps 1e-12).
    # The same scenario blocks as the headline.
    x_s = torch.zeros_like(b_d)

    def spec_step():
        if blk is not None:
            blk.step(blk_a, blk_b, blk_x, tol=1e-10, max_sweeps=IR_MAX_SWEEPS, sweeps=blk_sw,
                     stream=stream)
        else:
            num.scatter_refactor(a_d, stream=stream)
            num.solve_refined(a_d, b_d, x_s, tol=1e-10, max_sweeps=IR_MAX_SWEEPS,
                              sweeps=sweeps, stream=stream)

    for _ in range(args.warmup):
        spec_step()
    if blk is not None:
        ms_s = _time_blocks_ms(blk, (blk_a, blk_b, blk_x),
                               {"tol": 1e-10, "max_sweeps": IR_MAX_SWEEPS, "sweeps": blk_sw},
                               stream, args.steps)
    else:
        ms_s = _time_ms(spec_step, stream, args.steps)
    if blk is not None:
        Hb = S // n_blk
        sw_s = np.concatenate([t.cpu().numpy()[:Hb] for t in blk_sw])
        xs_h = np.concatenate([t.cpu().numpy()[:, :Hb] for t in blk_x], axis=1)
    else:
        sw_s = sweeps.cpu().numpy()[:S]
        xs_h = x_s.cpu().numpy()[:, :S]
    spec_oracle = []
    for k in sorted({0, 1, S // 3, S // 2, (2 * S) // 3, S - 1}):
        _, x_ref = port.scatter_refactor_solve(a[:, k], b[:, k])
        spec_oracle.append(float(np.abs(xs_h[:, k] - x_ref).max() / np.abs(x_ref).max()))
    at_spec_tolerance = {
        "value": S / (ms_s / 1000.0), "unit": UNIT, "ms_per_step": ms_s, "ir_tol": 1e-10,
        "sweeps_min": int(sw_s.min()), "sweeps_max": int(sw_s.max()),
        "not_converged": int((sw_s <= 0).sum()),
        "max_rel_err_vs_fp64": float(np.max(np.abs(xs_h - xb).max(axis=0) /
                                            np.abs(xb).max(axis=0))),
        "max_rel_err_vs_oracle_fp64": max(spec_oracle)}
    del x_s

    # Plain single-instance FP64 GPU path: one scenario, scatter + refactor +
    # solve, in each schedule; the fastest is the denominator of the ratio.
    a1 = a_d[:, 0].contiguous()
    b1 = b_d[:, 0].contiguous()
    x1 = b1.clone()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    plain_iters = 200
    single = {}
    plain_tuning = None
    for name, sched in (("thread_chain_levels", SCHED_THREAD_CHAIN),
                        ("programs_levels", SCHED_LEVELS),
                        ("programs_persistent", SCHED_PERSISTENT),
                        ("programs_autotuned", None)):
        if sched is None:
            plain_tuning, _ = _autotune(sym, 1, FP64)
            one = Numeric(sym, 1, FP64, tuning=plain_tuning)
        else:
            one = Numeric(sym, 1, FP64, sched)

        def plain_step():
            one.scatter(a1, stream=stream)
            x1.copy_(b1)
            one.refactor_solve(x1, original=True, stream=stream)

        for _ in range(5):
            plain_step()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(plain_iters):
            plain_step()
        e1.record(stream)
        torch.cuda.synchronize()
        single[name] = plain_iters / (e0.elapsed_time(e1) / 1000.0)
        del one
    plain_name = max(single, key=single.get)
    plain = single[plain_name]

    # The same 512-scenario batch in FP64 (scatter + FP64 refactor + solve,
    # autotuned), which splits the headline's gain over the plain path into
    # the part that batching gives and the part that FP32 + refinement adds.
    from phdthesis_albertojimenezruiz_gb300.glu import autotune_ex

    t64, _ = _autotune(sym,S, FP64)
    num64b = Numeric(sym, S, FP64, tuning=t64)
    x64b = torch.empty_like(b_d)

    def fp64_step():
        if t64["schedule"] == SCHED_LEVELS:  # scatter + refactor in one pass
            num64b.scatter_refactor(a_d, stream=stream)
            x64b.copy_(b_d)
            num64b.solve(x64b, original=True, stream=stream)
        else:  # refactor + solve in one persistent launch
            num64b.scatter(a_d, stream=stream)
            x64b.copy_(b_d)
            num64b.refactor_solve(x64b, original=True, stream=stream)

    for _ in range(args.warmup):
        fp64_step()
    ms64 = _time_ms(fp64_step, stream, args.steps)
    batched_fp64 = {"value": S / (ms64 / 1000.0), "unit": UNIT, "ms_per_step": ms64,
                    "tuning": t64,
                    "max_rel_err_vs_fp32ir": float(np.max(
                        np.abs(x64b.cpu().numpy()[:, :S] - xa).max(axis=0) /
                        np.abs(xa).max(axis=0)))}
    if blk is not None and t64["schedule"] == SCHED_LEVELS:
        # The FP64 step as the headline's scenario blocks too.
        blk64 = Blocks(sym, S, n_blk, FP64, tuning={k: t64[k] for k in tuning})
        x64k = [torch.empty_like(t) for t in blk_b]

        def fp64_block_step():
            blk64.step(blk_a, blk_b, x64k, stream=stream)

        for _ in range(args.warmup):
            fp64_block_step()
        ms64k = _time_blocks_ms(blk64, (blk_a, blk_b, x64k), {}, stream, args.steps)
        Hb = S // n_blk
        same64 = all(torch.equal(x64k[k][:, :Hb], x64b[:, k * Hb:(k + 1) * Hb])
                     for k in range(n_blk))
        batched_fp64["blocks"] = {"value": S / (ms64k / 1000.0), "unit": UNIT,
                                  "ms_per_step": ms64k, "blocks": n_blk,
                                  "bit_identical_to_one_handle": bool(same64)}
        del blk64, x64k
    del num64b, x64b

    # The same batched step with the reference's own AMD ordering of this
    # plant (a fixture made by the reference's code): its fill, levels and
    # rate beside the built-in ordering's.
    reference_ordering = None
    amd = ROOT / "tests" / "golden" / "orderings" / "plant_amd.npz"
    tag = "x".join(map(str, p.dims))
    if amd.exists():
        with np.load(amd) as z:
            perm = z[f"perm_{tag}"] if f"perm_{tag}" in z else None
        if perm is not None:
            sym_r = Symbolic(p.rowptr, p.colidx, perm)
            t_r, _ = _autotune(sym_r, S, FP32)
            num_r = Numeric(sym_r, S, FP32, tuning=t_r)
            x_r = torch.zeros_like(b_d)

            def ref_order_step():
                num_r.scatter_refactor(a_d, stream=stream)
                num_r.solve_refined(a_d, b_d, x_r, tol=IR_TOL, max_sweeps=IR_MAX_SWEEPS,
                                    sweeps=sweeps, stream=stream)

            for _ in range(args.warmup):
                ref_order_step()
            ms_r = _time_ms(ref_order_step, stream, args.steps)
            sw_r = sweeps.cpu().numpy()[:S]
            xr = x_r.cpu().numpy()[:, :S]
            reference_ordering = {
                "value": S / (ms_r / 1000.0), "unit": UNIT, "ms_per_step": ms_r,
                "ordering": "the reference's AMD ordering (004a), fixture "
                            "tests/golden/orderings/plant_amd.npz",
                "nnz_lu": int(sym_r.nnz_lu), "lu_levels": sym_r.info["lu_levels"],
                "u_levels": sym_r.info["u_levels"], "tuning": t_r,
                "sweeps_max": int(sw_r.max()), "not_converged": int((sw_r <= 0).sum()),
                "max_rel_err_vs_fp64": float(np.max(np.abs(xr - xb).max(axis=0) /
                                                    np.abs(xb).max(axis=0)))}
            del num_r, x_r

    # End to end through the host-buffer C ABI call: every step copies its
    # inputs from pinned host memory and its solutions back.  Two handles on
    # two streams alternate, so one batch's copies overlap the other's
    # kernels (the C2C link and the SMs work at the same time).
    a_h = torch.from_numpy(a).pin_memory()
    b_h = torch.from_numpy(b).pin_memory()
    x_hs = [torch.empty_like(b_h).pin_memory() for _ in range(2)]
    num2 = Numeric(sym, S, FP32, tuned["schedule"], max_locals=tuned["max_locals"])
    stream2 = torch.cuda.Stream()
    sweeps2 = torch.zeros(ld, dtype=torch.int32, device=dev)
    lanes = [(num, stream, sweeps), (num2, stream2, sweeps2)]
    for k in range(4):
        h_, st_, sw_ = lanes[k % 2]
        h_.refine_system_host(a_h, b_h, x_hs[k % 2], IR_TOL, IR_MAX_SWEEPS, sw_, stream=st_)
    torch.cuda.synchronize()
    e2e_steps = max(4, args.steps)
    if dist:
        dist.barrier()
    e2 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    stream2.wait_event(e0)
    for k in range(e2e_steps):
        h_, st_, sw_ = lanes[k % 2]
        h_.refine_system_host(a_h, b_h, x_hs[k % 2], IR_TOL, IR_MAX_SWEEPS, sw_, stream=st_)
    e2.record(stream2)
    stream.wait_event(e2)
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = max_over_ranks(e0.elapsed_time(e1), dist, dev)
    e2e = S * world * e2e_steps / (e2e_ms / 1000.0)
    e2e_sw = np.concatenate([sweeps.cpu().numpy()[:S], sweeps2.cpu().numpy()[:S]])
    e2e_err = float(np.max(np.abs(x_hs[0].numpy()[:, :S] - xb).max(axis=0) /
                           np.abs(xb).max(axis=0)))

    # The same end to end with the Jacobian as element conductances
    # (pvglu_refine_stamps_host): n_panels values per scenario cross the host
    # link instead of nnz_a.  Not the reference's interface (its hot path
    # takes assembled values); reported beside `e2e`.
    gpan = make_conductances(p, S, ld, seed0=1000 + rank * S)
    g_h = torch.from_numpy(gpan).pin_memory()
    for h_ in (num, num2):
        h_.set_stamps(p.n_panels, p.a_lin, p.contrib_ptr, p.contrib_panel, p.contrib_sign)
    for k in range(4):
        h_, st_, sw_ = lanes[k % 2]
        h_.refine_stamps_host(g_h, b_h, x_hs[k % 2], IR_TOL, IR_MAX_SWEEPS, sw_, stream=st_)
    torch.cuda.synchronize()
    es0 = torch.cuda.Event(enable_timing=True)
    es1 = torch.cuda.Event(enable_timing=True)
    es2 = torch.cuda.Event(enable_timing=True)
    es0.record(stream)
    stream2.wait_event(es0)
    for k in range(e2e_steps):
        h_, st_, sw_ = lanes[k % 2]
        h_.refine_stamps_host(g_h, b_h, x_hs[k % 2], IR_TOL, IR_MAX_SWEEPS, sw_, stream=st_)
    es2.record(stream2)
    stream.wait_event(es2)
    es1.record(stream)
    torch.cuda.synchronize()
    e2s_ms = max_over_ranks(es0.elapsed_time(es1), dist, dev)
    e2s_sw = np.concatenate([sweeps.cpu().numpy()[:S], sweeps2.cpu().numpy()[:S]])
    e2e_structured = {
        "value": S * world * e2e_steps / (e2s_ms / 1000.0), "unit": UNIT,
        "h2d_bytes_per_step": int(g_h.numel() * 8 + b_h.numel() * 8),
        "d2h_bytes_per_step": int(x_hs[0].numel() * 8),
        "call": "pvglu_refine_stamps_host (panel conductances in, x out), two handles on two "
                "streams alternating",
        "sweeps_max": int(e2s_sw.max()), "not_converged": int((e2s_sw <= 0).sum()),
        "max_rel_err_vs_fp64": float(np.max(np.abs(x_hs[0].numpy()[:, :S] - xb).max(axis=0) /
                                            np.abs(xb).max(axis=0)))}
    del num2

    bm = bytes_model(nnz_a, nnz_lu, n, 4)
    peaks = _peaks()
    peak = peaks.get("hbm_gbs")
    # The per-level schedule scatters and refactors in one pass (without
    # WIDE levels, as on this plant); the persistent one scatters first.
    one_pass = not persistent and num.info["wide_levels"] == 0
    rf_bytes = bm["scatter_refactor"] if one_pass else bm["refactor"]
    achieved = rf_bytes * S / (refactor_ms / 1000.0) / 1e9
    roofline_refactor = {
        "kernel": ("k_prog_refactor_from_a<float> (scatter + refactor in one pass, both levels)"
                   if one_pass else "k_prog_persistent<float,batched> (refactor phase)"),
        "bound": "hbm",
        "achieved": achieved, "peak": peak, "unit": "GB/s",
        "frac": achieved / peak if peak else None,
        # DRAM read + write bytes of one scatter + refactorization (its two
        # level launches) from an ncu capture of this workload (512 scenarios).
        "traffic": REFACTOR_TRAFFIC_512 if S == 512 and one_pass else None,
        "peak_source": "measured" if peak else "fallback",
        "bytes_per_launch": rf_bytes * S, "avg_launch_ms": refactor_ms}
    achieved_r = bm["residual"] * S / (resid_ms / 1000.0) / 1e9
    roofline = {
        "kernel": "k_residual_rows (FP64 residual of the refinement, the largest share of a "
                  "step; one FP64 FMA per entry and scenario)",
        "bound": "hbm",
        "achieved": achieved_r, "peak": peak, "unit": "GB/s",
        "frac": achieved_r / peak if peak else None,
        # DRAM read + write bytes of one residual launch from an ncu capture
        # of this workload (512 scenarios).
        "traffic": RESIDUAL_TRAFFIC_512 if S == 512 else None,
        "peak_source": "measured" if peak else "fallback",
        "bytes_per_launch": bm["residual"] * S, "avg_launch_ms": resid_ms,
        "timing": "pvglu_refine_residual x20 (each with a 2 KB flag reset), CUDA events"}
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    extra = run_configs(args, stream)
    newton = (newton_section(p, sym, stream, args.newton_scenarios, 5000,
                             precision=args.newton_precision)
              if args.newton_scenarios > 0 else None)
    cpu = cpu_baseline(a[:, :S], b[:, :S], p, sym.array("perm_amd"), args.cpu_budget,
                       os.cpu_count() or 1, prefer_ref=True)
    # per step: scatter + refactor (one launch per level in one pass, else a
    # scatter first), permute b, then per sweep (all launched; converged work
    # exits at once) solve, update, check and residual.
    refactor_launches = 1 if persistent else sym.info["lu_levels"]
    solve_launches = 1 if persistent else sym.info["l_levels"] + sym.info["u_levels"]
    def handle_launches(sweeps_run: int) -> int:
        if persistent:  # sweep by sweep: every sweep up to the cap is launched
            refine = IR_MAX_SWEEPS * (solve_launches + 2) + IR_MAX_SWEEPS - 1
        else:  # graph: permute, first sweep, then residual + solve + update + check per sweep
            refine = 1 + (solve_launches + 2) + (sweeps_run - 1) * (solve_launches + 3)
        return (0 if one_pass else 1) + refactor_launches + refine

    if blk is not None:  # every block launches its own sequence
        launches = args.steps * sum(handle_launches(int(t[:S // n_blk].max().item()))
                                    for t in blk_sw)
    else:
        launches = args.steps * handle_launches(int(sw.max()))
    fp64_like = batched_fp64.get("blocks", batched_fp64)["value"]
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 LU + f64 refinement",
        "data": "synthetic (seeded Gaussian-shadow irradiance, flat-start companion Jacobians)",
        "config": {"workload": f"plant_{DIMS[0]}x{DIMS[1]}x{DIMS[2]} ({n} unknowns, nnz_a "
                               f"{nnz_a}, nnz_lu {nnz_lu}): scatter + FP32 GLU refactor + "
                               f"FP64-refined solve, {S} scenarios per step",
                   "scenarios_per_step": S, "parallelism": f"replicas x{world}",
                   "blocks": n_blk,
                   "call": (f"pvglu_blocks_step: {n_blk} blocks of {S // n_blk} scenarios, each "
                            "pvglu_scatter_refactor + pvglu_solve_refined on a stream of its own; "
                            "each block runs its steps back to back, joined after the last"
                            if n_blk > 1 else
                            "pvglu_scatter_refactor + pvglu_solve_refined"),
                   "l2": "inputs larger than L2 (FP64 Jacobian values "
                         f"{8 * nnz_a * ld / 1e6:.0f} MB per batch)",
                   "ir_tol": IR_TOL, "ir_max_sweeps": IR_MAX_SWEEPS, "tuning": tuned,
                   "flops_per_refactor_solve": sym.info["flops_refactor"] + 2.0 * nnz_lu},
        "ir": {"sweeps_min": int(sw.min()), "sweeps_max": int(sw.max()),
               "not_converged": int((sw <= 0).sum()), "max_rel_err_vs_fp64": max_rel,
               "max_rel_err_vs_oracle_fp64": max(oracle_err),
               "oracle_sample": f"{len(oracle_err)} scenarios"},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(8 * (nnz_a + n) * ld),
                "d2h_bytes_per_step": int(8 * n * ld),
                "call": "pvglu_refine_system_host, two handles on two streams alternating",
                "sweeps_max": int(e2e_sw.max()), "not_converged": int((e2e_sw <= 0).sum()),
                "max_rel_err_vs_fp64": e2e_err},
        "e2e_structured": e2e_structured,
        "single_handle": single_handle,
        "roofline": roofline,
        "roofline_refactor": roofline_refactor,
        "cpu_baseline": cpu,
        "newton_adjoint": newton,
        **extra,
        "gpu_launches": launches,
        "clocks": clk.summary(),
        # Last on the line, so that a tail of the output keeps them: the
        # target's denominator (the plain single-instance FP64 GPU path) and
        # the split of the headline into batching and precision.
        "at_spec_tolerance": at_spec_tolerance,
        "reference_ordering": reference_ordering,
        "batched_fp64": batched_fp64,
        "plain_fp64": {"value": plain, "unit": UNIT, "schedule": plain_name,
                       "all_schedules": single, "autotuned": plain_tuning},
        # Like for like: the batched FP64 step in the headline's form (its
        # scenario blocks where the headline uses them).
        "ratios": {"batched_fp32ir_over_plain_fp64": value / world / plain,
                   "batched_fp64_over_plain_fp64": fp64_like / plain,
                   "batched_fp32ir_over_batched_fp64": value / world / fp64_like,
                   "fp64_form": "scenario blocks" if "blocks" in batched_fp64 else "one handle"},
    }
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
