"""Python view of the pvglu C ABI.

`Symbolic` mirrors the reference's `prepare_matrices`
(PVPP_Plant_Simulator/000_PVPP_simulator.cpp:10-93) and exposes the arrays of
`struct_CPU_CUDA_arrays` (factorize_electrical_system.h:3-61).  `Numeric`
owns the device state and runs the hot path: `scatter` (fill_values_CSC_only,
010_create_CSR_CSC.cpp:142-155), `refactor` (factorize_electrical_system_CUDA,
factorize_electrical_system_CUDA.cu:61-152) and `solve`
(triangular_substitution_LU_CUDA, triangular_substitution.cu:232-271).
Device buffers are torch CUDA tensors passed by pointer; torch is plumbing
only, every computation runs in libpvglu.so.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N

SYMBOLIC_ARRAYS = (
    "perm_amd", "perm_rows", "row_orig", "col_orig", "fill_rowptr", "fill_col",
    "csr_rowptr", "csr_col", "csc_colptr", "csc_row", "csr_to_csc", "csc_to_csr",
    "csr_diag_start", "csc_diag_start", "lu_sl", "lu_sc", "lu_cols", "l_sl", "l_sc",
    "l_cols", "u_sl", "u_sc", "u_cols", "lt_sl", "lt_sc", "lt_cols",
    "max_elements_per_column", "slot_src", "diag_slot", "a_rowptr", "a_colidx",
)


def _stream_ptr(stream) -> C.c_void_p:
    if stream is None:
        return C.c_void_p(0)
    if isinstance(stream, int):
        return C.c_void_p(stream)
    return C.c_void_p(stream.cuda_stream)


def _ptr(t) -> C.c_void_p:
    if t is None:
        return C.c_void_p(0)
    if isinstance(t, np.ndarray):
        return C.c_void_p(t.ctypes.data)
    return C.c_void_p(t.data_ptr())


class Symbolic:
    """Host symbolic analysis of one Jacobian pattern (caller's unknown order)."""

    def __init__(self, rowptr, colidx, perm=None, _handle=None):
        if _handle is None:
            rowptr = np.ascontiguousarray(rowptr, dtype=np.int32)
            colidx = np.ascontiguousarray(colidx, dtype=np.int32)
            n = len(rowptr) - 1
            self._keep = [rowptr, colidx]
            p = None
            if perm is not None:
                p = np.ascontiguousarray(perm, dtype=np.int32)
                self._keep.append(p)
            h = C.c_void_p()
            N.check(N.lib().pvglu_symbolic_create(n, _ptr(rowptr), _ptr(colidx), _ptr(p),
                                                  C.byref(h)), "pvglu_symbolic_create")
        else:
            h = _handle
        self.handle = h
        info = N.SymbolicInfo()
        N.check(N.lib().pvglu_symbolic_get_info(h, C.byref(info)), "pvglu_symbolic_get_info")
        self.info = {f: getattr(info, f) for f, _ in N.SymbolicInfo._fields_}
        self.n = info.n
        self.nnz_a = info.nnz_a
        self.nnz_lu = info.nnz_lu

    def array(self, name: str) -> np.ndarray:
        ptr = C.POINTER(C.c_int)()
        ln = C.c_int64()
        N.check(N.lib().pvglu_symbolic_get_array(self.handle, name.encode(), C.byref(ptr),
                                                 C.byref(ln)), "pvglu_symbolic_get_array")
        if ln.value == 0:
            return np.zeros(0, dtype=np.int32)
        return np.ctypeslib.as_array(ptr, shape=(ln.value,)).copy()

    def arrays(self) -> dict[str, np.ndarray]:
        return {k: self.array(k) for k in SYMBOLIC_ARRAYS}

    def save(self, path) -> None:
        N.check(N.lib().pvglu_symbolic_save(self.handle, str(path).encode()),
                "pvglu_symbolic_save")

    @classmethod
    def load(cls, path) -> "Symbolic":
        h = C.c_void_p()
        N.check(N.lib().pvglu_symbolic_load(str(path).encode(), C.byref(h)),
                "pvglu_symbolic_load")
        return cls(None, None, _handle=h)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h and N._lib is not None:
            N.lib().pvglu_symbolic_destroy(h)
            self.handle = None


class Numeric:
    """Device LU state for `n_scenarios` Jacobians sharing one `Symbolic`."""

    def __init__(self, sym: Symbolic, n_scenarios: int = 1, precision: int = N.FP64,
                 schedule: int = N.SCHED_LEVELS, max_locals: int = 0, tuning: dict | None = None):
        """tuning (the dict of autotune_ex, pvglu_tuning's fields) overrides
        schedule and max_locals."""
        self.sym = sym
        h = C.c_void_p()
        if tuning is not None:
            t = N.Tuning(**{f: int(tuning[f]) for f, _ in N.Tuning._fields_})
            N.check(N.lib().pvglu_numeric_create_tuned(sym.handle, n_scenarios, precision,
                                                       C.byref(t), C.byref(h)),
                    "pvglu_numeric_create_tuned")
            schedule = t.schedule
        else:
            N.check(N.lib().pvglu_numeric_create_ex(sym.handle, n_scenarios, precision,
                                                    int(max_locals), C.byref(h)),
                    "pvglu_numeric_create_ex")
        self.max_locals = N.lib().pvglu_numeric_max_locals(h)
        self.handle = h
        self.S = n_scenarios
        self.ld = N.lib().pvglu_numeric_ld(h)
        self.precision = precision
        self.set_schedule(schedule)

    @property
    def info(self) -> dict:
        """pvglu_numeric_get_info: program levels, WIDE levels and units, widest
        table, chain-program operations and loads."""
        inf = N.NumericInfo()
        N.check(N.lib().pvglu_numeric_get_info(self.handle, C.byref(inf)),
                "pvglu_numeric_get_info")
        return {f: getattr(inf, f) for f, _ in N.NumericInfo._fields_}

    def set_schedule(self, schedule: int) -> None:
        N.check(N.lib().pvglu_numeric_set_schedule(self.handle, schedule),
                "pvglu_numeric_set_schedule")
        self.schedule = schedule

    def set_pivot_tol(self, tol: float) -> None:
        N.check(N.lib().pvglu_numeric_set_pivot_tol(self.handle, tol), "pvglu_numeric_set_pivot_tol")

    def values_ptr(self) -> int:
        return N.lib().pvglu_numeric_values(self.handle)

    def scatter(self, a_values, stream=None) -> None:
        N.check(N.lib().pvglu_scatter(self.handle, _ptr(a_values), _stream_ptr(stream)),
                "pvglu_scatter")

    def refactor(self, stream=None) -> None:
        N.check(N.lib().pvglu_refactor(self.handle, _stream_ptr(stream)), "pvglu_refactor")

    def scatter_refactor(self, a_values, stream=None) -> None:
        """pvglu_scatter_refactor: the factors of scatter() then refactor()."""
        N.check(N.lib().pvglu_scatter_refactor(self.handle, _ptr(a_values), _stream_ptr(stream)),
                "pvglu_scatter_refactor")

    def solve(self, x, transpose: bool = False, original: bool = False, stream=None) -> None:
        flags = (N.SOLVE_TRANSPOSE if transpose else 0) | (N.SOLVE_ORIGINAL if original else 0)
        N.check(N.lib().pvglu_solve(self.handle, _ptr(x), flags, _stream_ptr(stream)),
                "pvglu_solve")

    def refactor_solve(self, x, transpose: bool = False, original: bool = False,
                       stream=None) -> None:
        flags = (N.SOLVE_TRANSPOSE if transpose else 0) | (N.SOLVE_ORIGINAL if original else 0)
        N.check(N.lib().pvglu_refactor_solve(self.handle, _ptr(x), flags, _stream_ptr(stream)),
                "pvglu_refactor_solve")

    def solve_refined(self, a_values, b, x, tol=1e-12, max_sweeps=10, sweeps=None,
                      stream=None) -> None:
        N.check(N.lib().pvglu_solve_refined(self.handle, _ptr(a_values), _ptr(b), _ptr(x),
                                            float(tol), int(max_sweeps), _ptr(sweeps),
                                            _stream_ptr(stream)), "pvglu_solve_refined")

    def refine(self, b, x, a_values=None, g=None, gmin=None, transpose=False, tol=1e-12,
               max_sweeps=10, sweeps=None, stream=None) -> None:
        """pvglu_refine: J from explicit `a_values` or from the stamps over `g`."""
        flags = N.SOLVE_TRANSPOSE if transpose else 0
        N.check(N.lib().pvglu_refine(self.handle, _ptr(a_values), _ptr(g), _ptr(gmin), _ptr(b),
                                     _ptr(x), flags, float(tol), int(max_sweeps), _ptr(sweeps),
                                     _stream_ptr(stream)), "pvglu_refine")

    def set_stamps(self, n_elems: int, base, entry_ptr, entry_elem, entry_sign) -> None:
        """Registers a structured Jacobian (pvglu_numeric_set_stamps)."""
        self._stamps = [np.ascontiguousarray(base, dtype=np.float64),
                        np.ascontiguousarray(entry_ptr, dtype=np.int32),
                        np.ascontiguousarray(entry_elem, dtype=np.int32),
                        np.ascontiguousarray(entry_sign, dtype=np.int32)]
        N.check(N.lib().pvglu_numeric_set_stamps(self.handle, int(n_elems),
                                                 *[_ptr(a) for a in self._stamps]),
                "pvglu_numeric_set_stamps")

    def scatter_stamps(self, g, gmin=None, stream=None) -> None:
        N.check(N.lib().pvglu_scatter_stamps(self.handle, _ptr(g), _ptr(gmin),
                                             _stream_ptr(stream)), "pvglu_scatter_stamps")

    def check(self, stream=None) -> tuple[int, int, int]:
        code, col, sc = C.c_int(), C.c_int(), C.c_int()
        N.check(N.lib().pvglu_numeric_check(self.handle, _stream_ptr(stream), C.byref(code),
                                            C.byref(col), C.byref(sc)), "pvglu_numeric_check")
        return code.value, col.value, sc.value

    def refactor_host(self, csc_values: np.ndarray) -> None:
        N.check(N.lib().pvglu_refactor_host(self.handle, _ptr(csc_values)), "pvglu_refactor_host")

    def solve_host(self, b: np.ndarray) -> None:
        N.check(N.lib().pvglu_solve_host(self.handle, _ptr(b)), "pvglu_solve_host")

    def scatter_refactor_solve_host(self, a_values, b, x, stream=None) -> None:
        N.check(N.lib().pvglu_scatter_refactor_solve_host(self.handle, _ptr(a_values), _ptr(b),
                                                          _ptr(x), _stream_ptr(stream)),
                "pvglu_scatter_refactor_solve_host")

    def refine_residual(self, a_values, b, x, r, stream=None) -> None:
        """r = b - J x (FP64 arithmetic) rounded to FP32, pivot order: one
        residual of the refinement (FP32 handles)."""
        N.check(N.lib().pvglu_refine_residual(self.handle, _ptr(a_values), _ptr(b), _ptr(x),
                                              _ptr(r), _stream_ptr(stream)),
                "pvglu_refine_residual")

    def refine_system_host(self, a_values, b, x, tol=1e-12, max_sweeps=10, sweeps=None,
                           stream=None) -> None:
        N.check(N.lib().pvglu_refine_system_host(self.handle, _ptr(a_values), _ptr(b), _ptr(x),
                                                 float(tol), int(max_sweeps), _ptr(sweeps),
                                                 _stream_ptr(stream)),
                "pvglu_refine_system_host")

    def refine_stamps_host(self, g, b, x, tol=1e-12, max_sweeps=10, sweeps=None,
                           stream=None) -> None:
        """Host-buffer refined step with the Jacobian from the registered
        stamps: element conductances g [n_elems x ld] in, x out."""
        N.check(N.lib().pvglu_refine_stamps_host(self.handle, _ptr(g), _ptr(b), _ptr(x),
                                                 float(tol), int(max_sweeps), _ptr(sweeps),
                                                 _stream_ptr(stream)),
                "pvglu_refine_stamps_host")

    def __del__(self):
        h = getattr(self, "handle", None)
        if h and N._lib is not None and getattr(self, "_owned", True):
            N.lib().pvglu_numeric_destroy(h)
            self.handle = None

    @classmethod
    def _borrow(cls, sym: Symbolic, handle: C.c_void_p, n_scenarios: int,
                precision: int) -> "Numeric":
        """A view of a handle owned elsewhere (a block of Blocks)."""
        self = cls.__new__(cls)
        self._owned = False
        self.sym = sym
        self.handle = handle
        self.S = n_scenarios
        self.ld = N.lib().pvglu_numeric_ld(handle)
        self.max_locals = N.lib().pvglu_numeric_max_locals(handle)
        self.precision = precision
        self.schedule = None
        return self


class Blocks:
    """One batch of scenarios as `parts` numeric handles of n_scenarios /
    parts scenarios, run side by side on streams of their own
    (pvglu_blocks_*).  Block k's buffers have the layout of parts[k]."""

    def __init__(self, sym: Symbolic, n_scenarios: int, parts: int, precision: int = N.FP32,
                 tuning: dict | None = None):
        h = C.c_void_p()
        t = None
        if tuning is not None:
            t = N.Tuning(**{f: int(tuning[f]) for f, _ in N.Tuning._fields_})
        N.check(N.lib().pvglu_blocks_create(sym.handle, int(n_scenarios), int(parts),
                                            int(precision), C.byref(t) if t else None,
                                            C.byref(h)), "pvglu_blocks_create")
        self.handle = h
        self.sym = sym
        self.S = n_scenarios
        self.precision = precision
        self.parts = []
        for k in range(parts):
            hk = C.c_void_p()
            N.check(N.lib().pvglu_blocks_part(h, k, C.byref(hk)), "pvglu_blocks_part")
            self.parts.append(Numeric._borrow(sym, hk, n_scenarios // parts, precision))

    def step(self, a_values, b, x, tol=1e-12, max_sweeps=10, sweeps=None, stream=None,
             join: bool = True) -> None:
        """pvglu_blocks_step: per block k, factors from a_values[k] and
        x[k] = J^-1 b[k] (refined to tol for FP32 blocks).  join=False: the
        stream does not wait for the blocks (see join())."""
        n = len(self.parts)

        def arr(bufs):
            return (C.c_void_p * n)(*[_ptr(t).value for t in bufs])

        sw = None if sweeps is None else arr(sweeps)
        flags = 0 if join else N.BLOCKS_NO_JOIN
        N.check(N.lib().pvglu_blocks_step(self.handle, arr(a_values), arr(b), arr(x), float(tol),
                                          int(max_sweeps), sw, flags, _stream_ptr(stream)),
                "pvglu_blocks_step")

    def join(self, stream=None) -> None:
        """pvglu_blocks_join: the stream waits for every block's work so far."""
        N.check(N.lib().pvglu_blocks_join(self.handle, _stream_ptr(stream)), "pvglu_blocks_join")

    def __del__(self):
        h = getattr(self, "handle", None)
        if h and N._lib is not None:
            for p in getattr(self, "parts", []):
                p.handle = None
            N.lib().pvglu_blocks_destroy(h)
            self.handle = None


class Group:
    """Numeric handles of different size classes refactored and solved
    together, one launch per level (pvglu_group_*)."""

    def __init__(self, members: list[Numeric]):
        self.members = list(members)
        arr = (C.c_void_p * len(members))(*[m.handle.value for m in members])
        h = C.c_void_p()
        N.check(N.lib().pvglu_group_create(arr, len(members), C.byref(h)), "pvglu_group_create")
        self.handle = h

    def refactor_solve(self, xs=None, original: bool = False, stream=None) -> None:
        arr = None
        if xs is not None:
            arr = (C.c_void_p * len(xs))(*[_ptr(x).value for x in xs])
        flags = N.SOLVE_ORIGINAL if original else 0
        N.check(N.lib().pvglu_group_refactor_solve(self.handle, arr, flags, _stream_ptr(stream)),
                "pvglu_group_refactor_solve")

    def __del__(self):
        h = getattr(self, "handle", None)
        if h and N._lib is not None:
            N.lib().pvglu_group_destroy(h)
            self.handle = None


def autotune(sym: Symbolic, n_scenarios: int, precision: int) -> tuple[int, int, float]:
    """pvglu_autotune: (max_locals, schedule, ms per scatter+refactor+solve)."""
    ml, sc, ms = C.c_int(), C.c_int(), C.c_double()
    N.check(N.lib().pvglu_autotune(sym.handle, int(n_scenarios), int(precision), C.byref(ml),
                                   C.byref(sc), C.byref(ms)), "pvglu_autotune")
    return ml.value, sc.value, ms.value


def autotune_ex(sym: Symbolic, n_scenarios: int, precision: int) -> tuple[dict, float]:
    """pvglu_autotune_ex: (tuning dict for Numeric(tuning=...), ms per
    scatter+refactor+solve)."""
    t = N.Tuning()
    ms = C.c_double()
    N.check(N.lib().pvglu_autotune_ex(sym.handle, int(n_scenarios), int(precision), C.byref(t),
                                      C.byref(ms)), "pvglu_autotune_ex")
    return {f: getattr(t, f) for f, _ in N.Tuning._fields_}, ms.value


# Names of the reference's entry points, for callers porting a driver.
def prepare_matrices(rowptr, colidx, perm=None) -> Symbolic:
    """prepare_matrices (000_PVPP_simulator.cpp:10-93)."""
    return Symbolic(rowptr, colidx, perm)


def factorize_electrical_system_CUDA(num: Numeric, stream=None) -> None:  # noqa: N802
    """factorize_electrical_system_CUDA (factorize_electrical_system_CUDA.cu:61-152)."""
    num.refactor(stream)


def triangular_substitution_LU_CUDA(num: Numeric, solution, stream=None) -> None:  # noqa: N802
    """triangular_substitution_LU_CUDA (triangular_substitution.cu:232-271); permuted space."""
    num.solve(solution, stream=stream)
