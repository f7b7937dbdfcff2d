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


def block_plant(blocks: int, strings: int, panels: int, seed: int = 0):
    """A Jacobian with the reference simulator's own plant topology
    (PVPP_Plant_Simulator/003_create_electric_system.cpp:89-126, 184-262,
    264-342; interconnection "nothing"): per block, `strings` series strings
    of `panels` panels in parallel between two bus nodes; every panel has an
    internal diode node with its series and shunt resistors and its diode;
    the buses reach the block's inverter (a DC voltage source with its own
    current unknown) through wires, one bus is grounded through a wire; per
    block two AC phasor nodes (real and imaginary unknowns) on a ring of AC
    wires closed at the point of common coupling, an AC voltage source.  The
    inverters' AC injections are right-hand-side terms only (002b:205-237),
    so they add no entries.  Unknowns in the reference's order: nodes in
    creation order, then the voltage-source currents.

    Eliminating a string from its bus end fills the bus rows and columns
    with an entry per string node, so the factors have a few dense columns
    and rows (about strings x panels entries each) and long dependency
    chains: the shape the reference's own plant gives its GLU.

    Values are this function's own (the reference's Rs = 0.115 ohm, Rsh =
    90.85 ohm and 1e-5 ohm wires; seeded diode conductances of a forward-
    biased operating point).  Returns (rowptr, colidx, values, b) in CSR.
    """
    rng = np.random.default_rng(seed)
    g_rs, g_rsh, g_wire = 1.0 / 0.115, 1.0 / 90.85, 1.0 / 1e-5
    entries: dict[tuple[int, int], float] = {}
    n_nodes = 0

    def node() -> int:  # 1-based node number, 0 = ground
        nonlocal n_nodes
        n_nodes += 1
        return n_nodes

    def add(r: int, c: int, v: float) -> None:
        entries[(r, c)] = entries.get((r, c), 0.0) + v

    def adm(n1: int, n2: int, g: float) -> None:
        if n1:
            add(n1 - 1, n1 - 1, g)
        if n1 and n2:
            add(n1 - 1, n2 - 1, -g)
            add(n2 - 1, n1 - 1, -g)
        if n2:
            add(n2 - 1, n2 - 1, g)

    def adm_ac(n1: int, n2: int, g: float) -> None:
        # 2x2 real blocks [Re -Im; Im Re] of a complex admittance g + 0j
        # (002b:41-67): the imaginary entries are stamped with zero.
        for a_, b_, s in ((n1, n1, 1.0), (n1, n2, -1.0), (n2, n1, -1.0), (n2, n2, 1.0)):
            if not a_ or not b_:
                continue
            r, c = a_ - 1, b_ - 1
            add(r, c, s * g)
            add(r, c + 1, 0.0)
            add(r + 1, c, 0.0)
            add(r + 1, c + 1, s * g)

    sources = []  # (n+, n-, value)
    rhs_nodes = []  # (node, value) current sources into the node
    mains = []
    for _ in range(blocks):
        bus_in, bus_out = node(), node()
        for _ in range(strings):
            hi_prev = None
            for j in range(panels):
                hi = bus_in if j == panels - 1 else node()
                lo = bus_out if j == 0 else hi_prev
                hi_prev = hi
                internal = node()
                adm(internal, hi, g_rs)
                adm(internal, lo, g_rsh)
                adm(internal, lo, float(rng.uniform(1e-4, 2.0)))  # diode companion G
                adm(lo, hi, float(rng.uniform(1e-9, 1e-6)))  # reverse-biased bypass diode
                rhs_nodes.append((internal, 8.5))
                rhs_nodes.append((lo, -8.5))
        after_in, after_out = node(), node()
        adm(after_in, bus_in, g_wire)
        adm(after_out, bus_out, g_wire)
        m0 = node()
        node()
        m1 = node()
        node()
        mains.append((m0, m1))
        adm(after_out, 0, g_wire)
        sources.append((after_in, after_out, 0.8 * 46.0 * panels))
        if len(mains) > 1:
            adm_ac(mains[-1][0], mains[-2][0], g_wire)
            adm_ac(mains[-1][1], mains[-2][1], g_wire)
    pcc = node()
    node()
    sources.append((pcc, 0, 25000.0))
    sources.append((pcc + 1, 0, 0.0))
    adm_ac(pcc, mains[0][0], g_wire)
    adm_ac(0, mains[0][1], g_wire)
    adm_ac(pcc, mains[-1][0], g_wire)
    adm_ac(0, mains[-1][1], g_wire)
    n = n_nodes + len(sources)
    b = np.zeros(n)
    for k, (p_, m_, val) in enumerate(sources):
        row = n_nodes + k
        if p_:
            add(p_ - 1, row, -1.0)
            add(row, p_ - 1, 1.0)
        if m_:
            add(m_ - 1, row, 1.0)
            add(row, m_ - 1, -1.0)
        b[row] += val
    for nd, val in rhs_nodes:
        b[nd - 1] += val
    keys = np.array(list(entries.keys()), dtype=np.int64)
    vals = np.array(list(entries.values()), dtype=np.float64)
    order = np.lexsort((keys[:, 1], keys[:, 0]))
    keys, vals = keys[order], vals[order]
    rowptr = np.zeros(n + 1, np.int32)
    np.add.at(rowptr, keys[:, 0] + 1, 1)
    rowptr = np.cumsum(rowptr).astype(np.int32)
    return rowptr, keys[:, 1].astype(np.int32), vals, b


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

    def irradiance_batch(self, seeds, t: float = 0.0, preset: str = "c1") -> np.ndarray:
        """`irradiance` of every seed, [n_panels, len(seeds)], computed on the
        host's threads (the calls drop the GIL)."""
        import os
        from concurrent.futures import ThreadPoolExecutor

        seeds = list(seeds)
        out = np.empty((self.n_panels, len(seeds)))
        with ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
            for k, g in enumerate(ex.map(lambda sd: self.irradiance(sd, t, preset), seeds)):
                out[:, k] = g
        return out

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

        def run(lo: int, hi: int) -> int:  # element range [lo, hi): the call drops the GIL
            return N.lib().pvglu_plant_panel_iv(self.handle, hi - lo, _ptr(iph[lo:hi]),
                                                _ptr(v[lo:hi]), _ptr(cur[lo:hi]),
                                                _ptr(didv[lo:hi]))

        chunk = 1 << 18
        if len(v) <= chunk:
            N.check(run(0, len(v)), "pvglu_plant_panel_iv")
        else:
            import os
            from concurrent.futures import ThreadPoolExecutor

            bounds = [(lo, min(lo + chunk, len(v))) for lo in range(0, len(v), chunk)]
            with ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
                for rc in ex.map(lambda b: run(*b), bounds):
                    N.check(rc, "pvglu_plant_panel_iv")
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
        import scipy.sparse as sp

        npan, S = g_irr.shape
        ld = ld or S
        cur, didv = self.panel_iv(self.iph(g_irr).ravel(), v_panel.ravel())
        gpan = (-didv).reshape(npan, S)
        ieq = (-cur).reshape(npan, S) - gpan * v_panel
        if getattr(self, "_stamp_mats", None) is None:
            # entry <- panel conductances, node <- panel currents
            entry = np.repeat(np.arange(len(self.a_lin)), np.diff(self.contrib_ptr))
            node = np.repeat(np.arange(self.n), np.diff(self.inc_ptr))
            self._stamp_mats = (
                sp.csr_matrix((self.contrib_sign.astype(np.float64), (entry, self.contrib_panel)),
                              shape=(len(self.a_lin), npan)),
                sp.csr_matrix((-self.inc_sign.astype(np.float64), (node, self.inc_panel)),
                              shape=(self.n, npan)))
        ma, mb = self._stamp_mats
        gst = gpan + gmin if gmin > 0 else gpan
        a = np.zeros((len(self.a_lin), ld))
        a[:, :S] = self.a_lin[:, None] + ma @ gst
        b = np.zeros((self.n, ld))
        b[:, :S] = self.b_lin[:, None] + mb @ ieq
        return a, b

    def __del__(self):
        h = getattr(self, "handle", None)
        if h and N._lib is not None:
            N.lib().pvglu_plant_destroy(h)
            self.handle = None
