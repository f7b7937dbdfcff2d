"""ctypes binding of libpvglu.so (include/pvglu.h, include/pvglu_plant.h,
include/pvglu_newton.h).

Loading fails loudly when the native library is missing: there is no Python
or CPU fallback for any hot-path operation.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_LIB_PATH = Path(__file__).resolve().parent / "libpvglu.so"

OK = 0
ERR_NAMES = {
    0: "OK", 1: "BAD_ARG", 2: "STRUCTURAL", 3: "ZERO_PIVOT", 4: "NONFINITE", 5: "CUDA",
    6: "BARRIER_TIMEOUT", 7: "NOT_CONVERGED", 8: "NO_MEMORY", 9: "TOO_LARGE",
}
FP64, FP32 = 0, 1
SOLVE_TRANSPOSE, SOLVE_ORIGINAL = 1, 2
BLOCKS_NO_JOIN = 1
SCHED_LEVELS, SCHED_PERSISTENT, SCHED_THREAD_CHAIN = 0, 1, 2
NEWTON_CONVERGED, NEWTON_RUNNING, NEWTON_MAX_ITERATIONS, NEWTON_DAMPING = 0, 1, 2, 3


class PvgluError(RuntimeError):
    def __init__(self, code: int, where: str, msg: str):
        super().__init__(f"{where}: {ERR_NAMES.get(code, code)} ({code}) {msg}")
        self.code = code


class SymbolicInfo(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("nnz_a", C.c_int64), ("nnz_lu", C.c_int64), ("update_count", C.c_int64),
        ("lu_levels", C.c_int), ("l_levels", C.c_int), ("u_levels", C.c_int), ("lt_levels", C.c_int),
        ("lu_chains", C.c_int), ("l_chains", C.c_int), ("u_chains", C.c_int), ("lt_chains", C.c_int),
        ("row_swaps", C.c_int), ("perm_rows_is_involution", C.c_int),
        ("right_looking_hazards", C.c_int64), ("flops_refactor", C.c_double),
    ]


class Tuning(C.Structure):
    _fields_ = [("max_locals", C.c_int), ("wide_threshold", C.c_int),
                ("merge_chains", C.c_int), ("schedule", C.c_int)]


class NumericInfo(C.Structure):
    _fields_ = [
        ("program_levels", C.c_int), ("wide_levels", C.c_int), ("wide_units", C.c_int),
        ("table_max", C.c_int), ("ops", C.c_int64), ("loads", C.c_int64),
    ]


class PlantInfo(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("n_panels", C.c_int), ("nnz_a", C.c_int64),
        ("n_inverters", C.c_int), ("n_strings", C.c_int), ("n_series", C.c_int),
        ("voc_panel", C.c_double), ("v_mppt", C.c_double), ("extent_x", C.c_double),
        ("extent_y", C.c_double), ("panel_i0", C.c_double), ("panel_a", C.c_double),
        ("panel_rs", C.c_double), ("panel_rsh", C.c_double), ("iph_stc", C.c_double),
    ]


class Circuit(C.Structure):
    _fields_ = [
        ("n_elems", C.c_int), ("elem_hi", C.c_void_p), ("elem_lo", C.c_void_p),
        ("a_lin", C.c_void_p), ("b_lin", C.c_void_p), ("i0", C.c_double), ("a", C.c_double),
        ("rs", C.c_double), ("rsh", C.c_double),
    ]


_P = C.c_void_p
_I = C.c_int
_IP = C.POINTER(C.c_int)
_DP = C.POINTER(C.c_double)

_SIGS = {
    "pvglu_last_error": ([], C.c_char_p),
    "pvglu_version": ([], C.c_char_p),
    "pvglu_symbolic_create": ([_I, _P, _P, _P, C.POINTER(_P)], _I),
    "pvglu_symbolic_destroy": ([_P], _I),
    "pvglu_symbolic_save": ([_P, C.c_char_p], _I),
    "pvglu_symbolic_load": ([C.c_char_p, C.POINTER(_P)], _I),
    "pvglu_symbolic_get_info": ([_P, C.POINTER(SymbolicInfo)], _I),
    "pvglu_symbolic_get_array": ([_P, C.c_char_p, C.POINTER(_IP), C.POINTER(C.c_int64)], _I),
    "pvglu_numeric_create": ([_P, _I, _I, C.POINTER(_P)], _I),
    "pvglu_numeric_create_ex": ([_P, _I, _I, _I, C.POINTER(_P)], _I),
    "pvglu_numeric_max_locals": ([_P], _I),
    "pvglu_numeric_get_info": ([_P, _P], _I),
    "pvglu_numeric_destroy": ([_P], _I),
    "pvglu_numeric_ld": ([_P], _I),
    "pvglu_numeric_values": ([_P], _P),
    "pvglu_numeric_set_schedule": ([_P, _I], _I),
    "pvglu_numeric_set_pivot_tol": ([_P, C.c_double], _I),
    "pvglu_scatter": ([_P, _P, _P], _I),
    "pvglu_scatter_refactor": ([_P, _P, _P], _I),
    "pvglu_refactor": ([_P, _P], _I),
    "pvglu_solve": ([_P, _P, _I, _P], _I),
    "pvglu_refactor_solve": ([_P, _P, _I, _P], _I),
    "pvglu_numeric_check": ([_P, _P, _IP, _IP, _IP], _I),
    "pvglu_refactor_host": ([_P, _P], _I),
    "pvglu_solve_host": ([_P, _P], _I),
    "pvglu_scatter_refactor_solve_host": ([_P, _P, _P, _P, _P], _I),
    "pvglu_solve_refined": ([_P, _P, _P, _P, C.c_double, _I, _P, _P], _I),
    "pvglu_selftest_barrier_timeout": ([_I, C.c_longlong, _IP, _IP], _I),
    "pvglu_autotune": ([_P, _I, _I, _IP, _IP, _DP], _I),
    "pvglu_autotune_ex": ([_P, _I, _I, _P, _DP], _I),
    "pvglu_numeric_create_tuned": ([_P, _I, _I, _P, _P], _I),
    "pvglu_group_create": ([_P, _I, C.POINTER(_P)], _I),
    "pvglu_blocks_create": ([_P, _I, _I, _I, _P, _P], _I),
    "pvglu_blocks_destroy": ([_P], _I),
    "pvglu_blocks_part": ([_P, _I, _P], _I),
    "pvglu_blocks_step": ([_P, _P, _P, _P, C.c_double, _I, _P, _I, _P], _I),
    "pvglu_blocks_join": ([_P, _P], _I),
    "pvglu_group_destroy": ([_P], _I),
    "pvglu_group_refactor_solve": ([_P, _P, _I, _P], _I),
    "pvglu_refine_system_host": ([_P, _P, _P, _P, C.c_double, _I, _P, _P], _I),
    "pvglu_refine_residual": ([_P, _P, _P, _P, _P, _P], _I),
    "pvglu_refine_stamps_host": ([_P, _P, _P, _P, C.c_double, _I, _P, _P], _I),
    "pvglu_solve_noalloc": ([_P, _P, _I, _P], _I),
    "pvglu_numeric_set_stamps": ([_P, _I, _P, _P, _P, _P], _I),
    "pvglu_scatter_stamps": ([_P, _P, _P, _P], _I),
    "pvglu_refine": ([_P, _P, _P, _P, _P, _P, _I, C.c_double, _I, _P, _P], _I),
    "pvglu_newton_create": ([_P, C.POINTER(Circuit), C.POINTER(_P)], _I),
    "pvglu_newton_destroy": ([_P], _I),
    "pvglu_newton_set_iph": ([_P, _P, _P], _I),
    "pvglu_newton_set_voltages": ([_P, _P, _P], _I),
    "pvglu_newton_set_refinement": ([_P, C.c_double, _I], _I),
    "pvglu_newton_set_broken": ([_P, _P, C.c_double], _I),
    "pvglu_newton_set_field": ([_P, _P, _P, _I, _P, _P, _P, C.c_double, C.c_double], _I),
    "pvglu_newton_field_iph": ([_P, C.c_double, _P, _P], _I),
    "pvglu_newton_run": ([_P, _P, _I, C.c_double, _I, _I, _P], _I),
    "pvglu_newton_results": ([_P, _P, _P, _P], _I),
    "pvglu_newton_voltages": ([_P], _P),
    "pvglu_newton_solution": ([_P, _P, _P], _I),
    "pvglu_newton_last_run": ([_P, _IP, _IP], _I),
    "pvglu_newton_adjoint": ([_P, _P, _P, _P], _I),
    "pvglu_newton_mismatch": ([_P, _P], _I),
    "pvglu_plant_create": ([_I, _I, _I, C.POINTER(_P)], _I),
    "pvglu_plant_destroy": ([_P], _I),
    "pvglu_plant_get_info": ([_P, C.POINTER(PlantInfo)], _I),
    "pvglu_plant_get_iarray": ([_P, C.c_char_p, C.POINTER(_IP), C.POINTER(C.c_int64)], _I),
    "pvglu_plant_get_darray": ([_P, C.c_char_p, C.POINTER(_DP), C.POINTER(C.c_int64)], _I),
    "pvglu_plant_irradiance": ([_P, _I, _I, C.c_double, C.c_double, C.c_uint64, C.c_double, _P], _I),
    "pvglu_plant_panel_iv": ([_P, _I, _P, _P, _P, _P], _I),
    "pvglu_plant_exp_log": ([_I, _P, _P, _P], _I),
    "pvglu_plant_shadows": ([_P, _I, _I, C.c_double, C.c_double, C.c_uint64, _IP, _P], _I),
}


def load_library(path: Path | None = None) -> C.CDLL:
    p = Path(path) if path else _LIB_PATH
    if not p.exists():
        raise ImportError(
            f"native library {p} is missing; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` (needs nvcc, sm_103a)")
    lib = C.CDLL(str(p))
    for name, (args, res) in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    return lib


_lib: C.CDLL | None = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        _lib = load_library()
    return _lib


def check(code: int, where: str) -> None:
    if code != OK:
        msg = lib().pvglu_last_error()
        raise PvgluError(code, where, msg.decode() if msg else "")


def exported_symbols() -> list[str]:
    return list(_SIGS)
