"""Synthetic PV plant (inverters x strings x series panels) and its Jacobians.

Thin view of include/pvglu_plant.h.  `jacobian_values` assembles the Newton
Jacobian of the companion model at given panel voltages on the host with
numpy, for tests and benchmarks that need realistic values; the device path
(Newton driver) assembles on the GPU.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .glu import _ptr

# Shadow presets of the synthetic configurations.
SHADOWS = {
    "c1": dict(min_shadows=3, max_shadows=3, min_depth=300.0, max_depth=800.0),
    "c2": dict(min_shadows=5, max_shadows=5, min_depth=300.0, max_depth=800.0),
    "c3": dict(min_shadows=3, max_shadows=8, min_depth=300.0, max_depth=800.0),
    "c4": dict(min_shadows=3, max_shadows=12, min_depth=300.0, max_depth=900.0),
}


class Plant:
    def __init__(self, n_inverters: int, n_strings: int, n_series: int):
        h = C.c_void_p()
        N.check(N.lib().pvglu_plant_create(n_inverters, n_strings, n_series, C.byref(h)),
                "pvglu_plant_create")
        self.handle = h
        info = N.PlantInfo()
        N.check(N.lib().pvglu_plant_get_info(h, C.byref(info)), "pvglu_plant_get_info")
        self.info = {f: getattr(info, f) for f, _ in N.PlantInfo._fields_}
        self.n = info.n
        self.n_panels = info.n_panels
        self.nnz_a = info.nnz_a
        self.v_mppt = info.v_mppt
        self.voc_panel = info.voc_panel
        self.n_series = n_series
        self.dims = (n_inverters, n_strings, n_series)
        for k in ("rowptr", "colidx", "pan_hi", "pan_lo", "contrib_ptr", "contrib_panel",
                  "contrib_sign", "inc_ptr", "inc_panel", "inc_sign", "inv_terminal",
                  "inv_current", "inv_combiner"):
            setattr(self, k, self._iarr(k))
        for k in ("a_lin", "b_lin", "pan_x", "pan_y"):
            setattr(self, k, self._darr(k))

    def _iarr(self, name):
        ptr = C.POINTER(C.c_int)()
        ln = C.c_int64()
        N.check(N.lib().pvglu_plant_get_iarray(self.handle, name.encode(), C.byref(ptr),
                                               C.byref(ln)), "pvglu_plant_get_iarray")
        return np.ctypeslib.as_array(ptr, shape=(ln.value,)).copy() if ln.value else np.zeros(0, np.int32)

    def _darr(self, name):
        ptr = C.POINTER(C.c_double)()
        ln = C.c_int64()
        N.check(N.lib().pvglu_plant_get_darray(self.handle, name.encode(), C.byref(ptr),
                                               C.byref(ln)), "pvglu_plant_get_darray")
        return np.ctypeslib.as_array(ptr, shape=(ln.value,)).copy() if ln.value else np.zeros(0)

    def irradiance(self, seed: int, t: float = 0.0, preset: str = "c1") -> np.ndarray:
        g = np.empty(self.n_panels)
        sh = SHADOWS[preset]
        N.check(N.lib().pvglu_plant_irradiance(self.handle, sh["min_shadows"], sh["max_shadows"],
                                               sh["min_depth"], sh["max_depth"], int(seed),
                                               float(t), _ptr(g)), "pvglu_plant_irradiance")
        return g

    def shadows(self, seed: int, preset: str = "c1") -> np.ndarray:
        """The seeded shadows of `irradiance(seed, t, preset)`: [count, 6] rows of
        (centre x, centre y, velocity x, velocity y, depth, sigma)."""
        sh = SHADOWS[preset]
        out = np.zeros((sh["max_shadows"], 6))
        cnt = C.c_int(0)
        N.check(N.lib().pvglu_plant_shadows(self.handle, sh["min_shadows"], sh["max_shadows"],
                                            sh["min_depth"], sh["max_depth"], int(seed),
                                            C.byref(cnt), _ptr(out)), "pvglu_plant_shadows")
        return out[: cnt.value].copy()

    def panel_iv(self, iph: np.ndarray, v: np.ndarray):
        iph = np.ascontiguousarray(iph, dtype=np.float64)
        v = np.ascontiguousarray(v, dtype=np.float64)
        cur = np.empty_like(v)
        didv = np.empty_like(v)
        N.check(N.lib().pvglu_plant_panel_iv(self.handle, len(v), _ptr(iph), _ptr(v), _ptr(cur),
                                             _ptr(didv)), "pvglu_plant_panel_iv")
        return cur, didv

    def iph(self, g: np.ndarray) -> np.ndarray:
        return self.info["iph_stc"] * g / 1000.0

    def inverter_block(self, v: int) -> tuple[slice, slice]:
        """Unknowns and panels of inverter v: (node slice, panel slice).

        The generator numbers the circuit inverter by inverter (the strings'
        panel nodes, then the combiner bus, the inverter terminal and the
        source current), and no element joins two inverters (each is a
        fixed-voltage sink), so block v of every array is the circuit of
        Plant(1, strings, series) shifted by v blocks."""
        per_node = self.dims[1] * self.dims[2] + 3
        per_pan = self.dims[1] * self.dims[2]
        return (slice(v * per_node, (v + 1) * per_node),
                slice(v * per_pan, (v + 1) * per_pan))

    def flat_start(self) -> np.ndarray:
        """Panel voltages of the flat start: every panel at V_mppt / n_series."""
        return np.full(self.n_panels, self.v_mppt / self.n_series)

    def jacobian_values(self, g_panel: np.ndarray) -> np.ndarray:
        """A-entry values (CSR order of `rowptr/colidx`) for panel conductances g."""
        counts = np.diff(self.contrib_ptr)
        contrib = self.contrib_sign * g_panel[self.contrib_panel]
        sums = np.zeros(len(self.a_lin))
        np.add.at(sums, np.repeat(np.arange(len(self.a_lin)), counts), contrib)
        return self.a_lin + sums

    def companion(self, g_irr: np.ndarray, v_panel: np.ndarray):
        """Companion model of every panel at voltage v: (G, Ieq, A values, b).

        Element current hi -> lo is f(V) = -I(V); G = f'(V), Ieq = f(V) - G V
        (002b_sistema_electrico_base_matriz.cpp:183-197)."""
        cur, didv = self.panel_iv(self.iph(g_irr), v_panel)
        gpan = -didv
        ieq = -cur - gpan * v_panel
        a = self.jacobian_values(gpan)
        b = self.b_lin.copy()
        np.add.at(b, np.repeat(np.arange(self.n), np.diff(self.inc_ptr)),
                  -self.inc_sign * ieq[self.inc_panel])
        return gpan, ieq, a, b

    def companion_batch(self, g_irr: np.ndarray, v_panel: np.ndarray, ld: int | None = None,
                        gmin: float = 0.0):
        """`companion` for S scenarios at once: g_irr, v_panel [n_panels, S].
        gmin > 0 adds the convergence conductance of a Newton stage to every
        panel's stamp (002b_sistema_electrico_base_matriz.cpp:198-202).

        Returns A values [nnz_a, ld] and b [n, ld] (columns past S zero)."""
        npan, S = g_irr.shape
        ld = ld or S
        cur, didv = self.panel_iv(self.iph(g_irr).ravel(), v_panel.ravel())
        gpan = (-didv).reshape(npan, S)
        ieq = (-cur).reshape(npan, S) - gpan * v_panel
        counts = np.diff(self.contrib_ptr)
        entry = np.repeat(np.arange(len(self.a_lin)), counts)
        a = np.zeros((len(self.a_lin), ld))
        a[:, :S] = self.a_lin[:, None]
        gst = gpan + gmin if gmin > 0 else gpan
        np.add.at(a[:, :S], entry, self.contrib_sign[:, None] * gst[self.contrib_panel])
        b = np.zeros((self.n, ld))
        b[:, :S] = self.b_lin[:, None]
        node = np.repeat(np.arange(self.n), np.diff(self.inc_ptr))
        np.add.at(b[:, :S], node, -self.inc_sign[:, None] * ieq[self.inc_panel])
        return a, b

    def __del__(self):
        h = getattr(self, "handle", None)
        if h and N._lib is not None:
            N.lib().pvglu_plant_destroy(h)
            self.handle = None
