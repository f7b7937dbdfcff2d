"""ORACLE — test infrastructure only.

ctypes loader for the CPU restatement (oracle/liboracle.so, built from
oracle_glu.cpp) and, where the reference checkout was available at build
time, for the reference's own code (oracle/_ref/libpvref.so, built by
oracle/Makefile.ref).  Only tests, the smoke check and bench.py's CPU legs use
this module; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
PORT_LIB = HERE / "liboracle.so"
REF_LIB = HERE / "_ref" / "libpvref.so"
# The reference checkout: $PVGLU_REFERENCE_DIR, by default a sibling
# "reference" directory of this repository.
REF_SRC = Path(os.environ.get("PVGLU_REFERENCE_DIR", str(ROOT.parent / "reference"))) / \
    "PVPP_Plant_Simulator"

ARRAYS = ("perm_amd", "perm_rows", "fill_rowptr", "fill_col", "lu_sl", "lu_sc", "lu_cols",
          "l_sl", "l_sc", "l_cols", "u_sl", "u_sc", "u_cols", "max_elements_per_column",
          "csr_rowptr", "csr_col", "csc_colptr", "csc_row", "csr_to_csc", "csc_to_csr",
          "csr_diag_start", "csc_diag_start")


def build_port() -> Path:
    subprocess.run(["make", "-s", "-f", str(HERE / "Makefile"), "oracle/liboracle.so"],
                   cwd=ROOT, check=True)
    return PORT_LIB


def build_ref() -> Path | None:
    """Builds oracle/_ref/libpvref.so when the reference sources are present."""
    if not REF_SRC.is_dir():
        return None
    subprocess.run(["make", "-s", "-j8", "-f", str(HERE / "Makefile.ref"), f"REF={REF_SRC}"],
                   cwd=ROOT, check=True)
    return REF_LIB


def _p(a):
    return C.c_void_p(0) if a is None else C.c_void_p(a.ctypes.data)


class _Base:
    prefix = ""

    def __init__(self, lib: C.CDLL, handle):
        self.lib = lib
        self.h = handle

    def get(self, name: str) -> np.ndarray:
        ptr = C.POINTER(C.c_int)()
        ln = C.c_longlong()
        rc = getattr(self.lib, self.prefix + "get")(self.h, name.encode(), C.byref(ptr), C.byref(ln))
        if rc:
            raise KeyError(name)
        if ln.value == 0:
            return np.zeros(0, np.int32)
        return np.ctypeslib.as_array(ptr, shape=(ln.value,)).copy()

    def arrays(self, names=ARRAYS) -> dict[str, np.ndarray]:
        return {k: self.get(k) for k in names}

    def scatter(self, a_vals: np.ndarray) -> np.ndarray:
        a = np.ascontiguousarray(a_vals, dtype=np.float64)
        out = np.empty(len(self.get("csc_row")))
        getattr(self.lib, self.prefix + "scatter")(self.h, _p(a), _p(out))
        return out

    def solve(self, lu: np.ndarray, b: np.ndarray) -> np.ndarray:
        x = np.array(b, dtype=np.float64, copy=True)
        lu = np.ascontiguousarray(lu, dtype=np.float64)  # keep alive across the call
        getattr(self.lib, self.prefix + "solve")(self.h, _p(lu), _p(x))
        return x

    def __del__(self):
        if getattr(self, "h", None):
            getattr(self.lib, self.prefix + "free")(self.h)
            self.h = None


class Port(_Base):
    """The CPU restatement in oracle_glu.cpp (P must be supplied)."""

    prefix = "oracle_"
    _lib = None

    @classmethod
    def lib_(cls):
        if cls._lib is None:
            if not PORT_LIB.exists():
                build_port()
            lib = C.CDLL(str(PORT_LIB))
            lib.oracle_symbolic.restype = C.c_void_p
            lib.oracle_symbolic.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.c_char_p, C.c_int]
            for f in ("oracle_get",):
                getattr(lib, f).argtypes = [C.c_void_p, C.c_char_p, C.c_void_p, C.c_void_p]
            for f in ("oracle_scatter", "oracle_solve", "oracle_solve_transposed"):
                getattr(lib, f).argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
            for f in ("oracle_refactor_levels", "oracle_refactor_sequential"):
                getattr(lib, f).argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
            lib.oracle_scatter_refactor_solve.argtypes = [C.c_void_p] * 4 + [C.c_int]
            D = C.c_double
            lib.oracle_newton.argtypes = ([C.c_void_p, C.c_int] + [C.c_void_p] * 4 + [C.c_int] +
                                          [C.c_void_p] * 2 + [D] * 4 + [C.c_void_p, D] +
                                          [C.c_void_p] * 3 + [C.c_int, D, C.c_int] +
                                          [C.c_void_p] * 3)
            lib.oracle_adjoint.argtypes = ([C.c_void_p, C.c_int] + [C.c_void_p] * 4 + [C.c_int] +
                                           [C.c_void_p] * 2 + [D] * 4 + [C.c_void_p, D] +
                                           [C.c_void_p] * 4)
            lib.oracle_fd_ext.argtypes = ([C.c_void_p, C.c_int] + [C.c_void_p] * 4 + [C.c_int] +
                                          [C.c_void_p] * 2 + [D] * 4 + [C.c_void_p] * 3 +
                                          [C.c_int, D, C.c_int] + [C.c_void_p] * 3)
            lib.oracle_free.argtypes = [C.c_void_p]
            cls._lib = lib
        return cls._lib

    def __init__(self, rowptr, colidx, perm):
        lib = self.lib_()
        self._keep = [np.ascontiguousarray(rowptr, dtype=np.int32),
                      np.ascontiguousarray(colidx, dtype=np.int32),
                      np.ascontiguousarray(perm, dtype=np.int32)]
        err = C.create_string_buffer(256)
        h = lib.oracle_symbolic(len(rowptr) - 1, _p(self._keep[0]), _p(self._keep[1]),
                                _p(self._keep[2]), err, 256)
        if not h:
            raise RuntimeError("oracle symbolic failed: " + err.value.decode())
        super().__init__(lib, h)

    def refactor(self, csc_vals: np.ndarray, sequential: bool = False) -> tuple[np.ndarray, int]:
        v = np.array(csc_vals, dtype=np.float64, copy=True)
        bad = C.c_int(-1)
        f = self.lib.oracle_refactor_sequential if sequential else self.lib.oracle_refactor_levels
        rc = f(self.h, _p(v), C.byref(bad))
        if rc:
            raise ZeroDivisionError(f"oracle pivot failure at column {bad.value}")
        return v

    def solve_transposed(self, lu: np.ndarray, b: np.ndarray) -> np.ndarray:
        x = np.array(b, dtype=np.float64, copy=True)
        lu = np.ascontiguousarray(lu, dtype=np.float64)
        self.lib.oracle_solve_transposed(self.h, _p(lu), _p(x))
        return x

    def scatter_refactor_solve(self, a_vals: np.ndarray, b: np.ndarray, sequential=True):
        """Scatter, refactor (sequential GLU by default: the valid LU on every
        pattern; level order reproduces the reference's level path), solve."""
        lu = np.empty(len(self.get("csc_row")))
        x = np.array(b, dtype=np.float64, copy=True)
        a = np.ascontiguousarray(a_vals, dtype=np.float64)
        rc = self.lib.oracle_scatter_refactor_solve(self.h, _p(a), _p(lu), _p(x),
                                                    1 if sequential else 0)
        if rc:
            raise ZeroDivisionError("oracle pivot failure")
        return lu, x


    # ---- Newton loop and adjoint (oracle_newton.cpp) -------------------------
    def _circuit(self, plant, broken=None, r_wire=1e-5):
        i = plant.info
        keep = [np.ascontiguousarray(plant.rowptr, dtype=np.int32),
                np.ascontiguousarray(plant.colidx, dtype=np.int32),
                np.ascontiguousarray(plant.a_lin, dtype=np.float64),
                np.ascontiguousarray(plant.b_lin, dtype=np.float64),
                np.ascontiguousarray(plant.pan_hi, dtype=np.int32),
                np.ascontiguousarray(plant.pan_lo, dtype=np.int32)]
        br = None if broken is None else np.ascontiguousarray(broken, dtype=np.int32)
        keep.append(br)
        args = [self.h, plant.n, _p(keep[0]), _p(keep[1]), _p(keep[2]), _p(keep[3]),
                plant.n_panels, _p(keep[4]), _p(keep[5]), i["panel_i0"], i["panel_a"],
                i["panel_rs"], i["panel_rsh"], _p(br), float(r_wire)]
        return keep, args

    def newton(self, plant, iph, v0, gmin, tol, max_iterations=5000, broken=None, r_wire=1e-5):
        """One scenario of the simulator's Newton loop (broken: panels
        replaced by a wire).  Returns (outcome, iterations, last diff, element
        voltages, node solution)."""
        keep, args = self._circuit(plant, broken, r_wire)
        iph = np.ascontiguousarray(iph, dtype=np.float64)
        v = np.array(v0, dtype=np.float64, copy=True)
        g = np.ascontiguousarray(gmin, dtype=np.float64)
        x = np.zeros(plant.n)
        it = C.c_int(0)
        diff = C.c_double(0.0)
        rc = self.lib.oracle_newton(*args, _p(iph), _p(v), _p(g), len(g), float(tol),
                                    int(max_iterations), _p(x), C.byref(it), C.byref(diff))
        del keep
        return rc, it.value, diff.value, v, x

    def adjoint(self, plant, iph, v, dpdx, broken=None, r_wire=1e-5):
        """dP/dIph per element at the iterate v for P = dpdx . x."""
        keep, args = self._circuit(plant, broken, r_wire)
        iph = np.ascontiguousarray(iph, dtype=np.float64)
        v = np.ascontiguousarray(v, dtype=np.float64)
        dpdx = np.ascontiguousarray(dpdx, dtype=np.float64)
        out = np.zeros(plant.n_panels)
        rc = self.lib.oracle_adjoint(*args, _p(iph), _p(v), _p(dpdx), _p(out))
        del keep
        if rc:
            raise RuntimeError(f"oracle adjoint failed ({rc})")
        return out

    def fd_ext(self, plant, iph, v0, dpdx, k, delta, max_iterations=40):
        """Central difference (P(iph_k + delta) - P(iph_k - delta)) / (2 delta)
        of P = dpdx . x, both operating points solved in long double from the
        element voltages v0 (oracle_fd_ext).  Returns (difference quotient,
        Newton iterations of the two sides, largest final residual [A])."""
        keep, args = self._circuit(plant)
        iph = np.ascontiguousarray(iph, dtype=np.float64)
        v0 = np.ascontiguousarray(v0, dtype=np.float64)
        dpdx = np.ascontiguousarray(dpdx, dtype=np.float64)
        fd = C.c_double(0.0)
        res = C.c_double(0.0)
        its = np.zeros(2, np.int32)
        rc = self.lib.oracle_fd_ext(*args[:13], _p(iph), _p(v0), _p(dpdx), int(k), float(delta),
                                    int(max_iterations), C.byref(fd), _p(its), C.byref(res))
        del keep
        if rc:
            raise RuntimeError(f"oracle extended-precision difference failed ({rc})")
        return fd.value, (int(its[0]), int(its[1])), res.value


class Ref(_Base):
    """The reference's own code (needs oracle/_ref/libpvref.so)."""

    prefix = "ref_"
    _lib = None

    @classmethod
    def available(cls) -> bool:
        return REF_LIB.exists()

    @classmethod
    def lib_(cls):
        if cls._lib is None:
            lib = C.CDLL(str(REF_LIB))
            lib.ref_symbolic.restype = C.c_void_p
            lib.ref_symbolic.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
            lib.ref_get.argtypes = [C.c_void_p, C.c_char_p, C.c_void_p, C.c_void_p]
            for f in ("ref_scatter", "ref_solve"):
                getattr(lib, f).argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
            for f in ("ref_refactor_levels", "ref_refactor_sequential"):
                getattr(lib, f).argtypes = [C.c_void_p, C.c_void_p]
            lib.ref_free.argtypes = [C.c_void_p]
            cls._lib = lib
        return cls._lib

    def __init__(self, rowptr, colidx, perm=None):
        lib = self.lib_()
        self._keep = [np.ascontiguousarray(rowptr, dtype=np.int32),
                      np.ascontiguousarray(colidx, dtype=np.int32)]
        p = None
        if perm is not None:
            p = np.ascontiguousarray(perm, dtype=np.int32)
            self._keep.append(p)
        h = lib.ref_symbolic(len(rowptr) - 1, _p(self._keep[0]), _p(self._keep[1]), _p(p))
        super().__init__(lib, h)

    def refactor(self, csc_vals: np.ndarray, sequential: bool = False) -> np.ndarray:
        v = np.array(csc_vals, dtype=np.float64, copy=True)
        f = self.lib.ref_refactor_sequential if sequential else self.lib.ref_refactor_levels
        f(self.h, _p(v))
        return v
