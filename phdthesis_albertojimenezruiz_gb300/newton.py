"""Device Newton driver of the PV plant (include/pvglu_newton.h).

`Newton` binds the damped, gmin-staged Newton iteration of the reference's
simulator (PVPP_Plant_Simulator/000_PVPP_simulator.cpp:163-236,
002b_sistema_electrico_base_matriz.cpp:141-240,
011_calculate_new_iteration.cpp:37-110) to a `Numeric` handle; every
iteration runs on the device (a CUDA graph where capture works) and the
adjoint gives dP/dIph for a linear objective P = dpdx . x.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .glu import Numeric, _ptr, _stream_ptr

# Convergence-conductance stages of the reference (000_PVPP_simulator.cpp:101-102).
GMIN_STAGES = (100.0, 10.0, 1.0, 0.9, 0.8, 0.5, 0.4, 0.3, 0.2, 0.1, 0.05, -1.0)
MAX_ITERATIONS = 5000  # 000_PVPP_simulator.cpp:152


class Newton:
    def __init__(self, num: Numeric, n_elems: int, elem_hi, elem_lo, a_lin, b_lin,
                 i0: float, a: float, rs: float, rsh: float):
        self.num = num
        self.n_elems = int(n_elems)
        self._keep = [np.ascontiguousarray(elem_hi, dtype=np.int32),
                      np.ascontiguousarray(elem_lo, dtype=np.int32),
                      np.ascontiguousarray(a_lin, dtype=np.float64),
                      np.ascontiguousarray(b_lin, dtype=np.float64)]
        c = N.Circuit(self.n_elems, *[k.ctypes.data for k in self._keep], float(i0), float(a),
                      float(rs), float(rsh))
        h = C.c_void_p()
        N.check(N.lib().pvglu_newton_create(num.handle, C.byref(c), C.byref(h)),
                "pvglu_newton_create")
        self.handle = h

    @classmethod
    def for_plant(cls, num: Numeric, plant) -> "Newton":
        i = plant.info
        return cls(num, plant.n_panels, plant.pan_hi, plant.pan_lo, plant.a_lin, plant.b_lin,
                   i["panel_i0"], i["panel_a"], i["panel_rs"], i["panel_rsh"])

    def set_iph(self, iph, stream=None) -> None:
        N.check(N.lib().pvglu_newton_set_iph(self.handle, _ptr(iph), _stream_ptr(stream)),
                "pvglu_newton_set_iph")

    def set_voltages(self, v, stream=None) -> None:
        N.check(N.lib().pvglu_newton_set_voltages(self.handle, _ptr(v), _stream_ptr(stream)),
                "pvglu_newton_set_voltages")

    def set_field(self, elem_x, elem_y, shadows_per_scenario, g_clear: float = 1000.0,
                  iph_per_g: float = 8.5 / 1000.0, t_offset=None) -> None:
        """Device irradiance field: one [count, 6] shadow array per scenario;
        t_offset [S]: scenario s sees the field at t + t_offset[s]."""
        mx = max([len(sh) for sh in shadows_per_scenario] + [1])
        S = len(shadows_per_scenario)
        counts = np.array([len(sh) for sh in shadows_per_scenario], dtype=np.int32)
        params = np.zeros((S, mx, 6))
        for s, sh in enumerate(shadows_per_scenario):
            params[s, : len(sh)] = sh
        toff = None if t_offset is None else np.ascontiguousarray(t_offset, dtype=np.float64)
        self._field = [np.ascontiguousarray(elem_x, dtype=np.float64),
                       np.ascontiguousarray(elem_y, dtype=np.float64), counts, params, toff]
        N.check(N.lib().pvglu_newton_set_field(self.handle, _ptr(self._field[0]),
                                               _ptr(self._field[1]), int(mx), _ptr(counts),
                                               _ptr(params), _ptr(toff), float(g_clear),
                                               float(iph_per_g)),
                "pvglu_newton_set_field")

    def field_iph(self, t: float, g_out=None, stream=None) -> None:
        N.check(N.lib().pvglu_newton_field_iph(self.handle, float(t), _ptr(g_out),
                                               _stream_ptr(stream)), "pvglu_newton_field_iph")

    def set_broken(self, broken=None, r_wire: float = 1e-5) -> None:
        """Flags [n_elems] of panels replaced by a wire (None clears)."""
        self._broken = None if broken is None else np.ascontiguousarray(broken, dtype=np.int32)
        N.check(N.lib().pvglu_newton_set_broken(self.handle, _ptr(self._broken), float(r_wire)),
                "pvglu_newton_set_broken")

    def set_refinement(self, tol: float, max_sweeps: int) -> None:
        N.check(N.lib().pvglu_newton_set_refinement(self.handle, float(tol), int(max_sweeps)),
                "pvglu_newton_set_refinement")

    def run(self, tol: float, gmin=GMIN_STAGES, max_iterations: int = MAX_ITERATIONS,
            check_every: int = 4, stream=None) -> None:
        g = np.ascontiguousarray(gmin, dtype=np.float64)
        N.check(N.lib().pvglu_newton_run(self.handle, _ptr(g), len(g), float(tol),
                                         int(max_iterations), int(check_every),
                                         _stream_ptr(stream)), "pvglu_newton_run")

    def results(self):
        S = self.num.S
        it = np.zeros(S, np.int32)
        out = np.zeros(S, np.int32)
        diff = np.zeros(S)
        N.check(N.lib().pvglu_newton_results(self.handle, _ptr(it), _ptr(out), _ptr(diff)),
                "pvglu_newton_results")
        return it, out, diff

    def last_run(self) -> tuple[int, bool]:
        bodies, graph = C.c_int(), C.c_int()
        N.check(N.lib().pvglu_newton_last_run(self.handle, C.byref(bodies), C.byref(graph)),
                "pvglu_newton_last_run")
        return bodies.value, bool(graph.value)

    def voltages_ptr(self) -> int:
        return N.lib().pvglu_newton_voltages(self.handle)

    def solution(self, x, stream=None) -> None:
        N.check(N.lib().pvglu_newton_solution(self.handle, _ptr(x), _stream_ptr(stream)),
                "pvglu_newton_solution")

    def mismatch(self) -> np.ndarray:
        """max_i |KCL mismatch| [A] per scenario at the node solution."""
        out = np.zeros(self.num.S)
        N.check(N.lib().pvglu_newton_mismatch(self.handle, _ptr(out)), "pvglu_newton_mismatch")
        return out

    def adjoint(self, dpdx, dpdiph, stream=None) -> None:
        N.check(N.lib().pvglu_newton_adjoint(self.handle, _ptr(dpdx), _ptr(dpdiph),
                                             _stream_ptr(stream)), "pvglu_newton_adjoint")

    def __del__(self):
        h = getattr(self, "handle", None)
        if h and N._lib is not None:
            N.lib().pvglu_newton_destroy(h)
            self.handle = None


def plant_power(newton: Newton, plant, g, tol: float = 1e-9, gmin=GMIN_STAGES):
    """Total MPPT power [W] of every scenario of `plant` at per-panel irradiance
    g (torch CUDA float64 [n_panels, S]), differentiable in g.

    Forward: the device Newton driver from the flat start (its factors and
    pattern stay in `newton`); backward: the adjoint (pvglu_newton_adjoint) at
    the converged operating point.  torch.autograd.Function semantics: the
    returned tensor has a grad_fn whose backward gives dP/dG."""
    import torch

    class _PlantPower(torch.autograd.Function):
        @staticmethod
        def forward(ctx, gg):
            num = newton.num
            ld, S = num.ld, num.S
            iph_per_g = plant.info["iph_stc"] / 1000.0
            iph = torch.zeros(plant.n_panels, ld, dtype=torch.float64, device=gg.device)
            iph[:, :S] = iph_per_g * gg
            v0 = torch.zeros_like(iph)
            v0[:, :S] = torch.as_tensor(plant.flat_start(), device=gg.device)[:, None]
            newton.set_iph(iph)
            newton.set_voltages(v0)
            newton.run(tol, gmin=gmin)
            x = torch.zeros(plant.n, ld, dtype=torch.float64, device=gg.device)
            newton.solution(x)
            cur = torch.as_tensor(plant.inv_current, dtype=torch.long, device=gg.device)
            ctx.iph_per_g = iph_per_g
            return -plant.v_mppt * x[cur, :S].sum(dim=0)

        @staticmethod
        def backward(ctx, grad_p):
            num = newton.num
            ld, S = num.ld, num.S
            dpdx = torch.zeros(plant.n, ld, dtype=torch.float64, device=grad_p.device)
            cur = torch.as_tensor(plant.inv_current, dtype=torch.long, device=grad_p.device)
            dpdx[cur, :S] = -plant.v_mppt * grad_p[None, :].to(torch.float64)
            out = torch.zeros(plant.n_panels, ld, dtype=torch.float64, device=grad_p.device)
            newton.adjoint(dpdx, out)
            return ctx.iph_per_g * out[:, :S]

    return _PlantPower.apply(g)
