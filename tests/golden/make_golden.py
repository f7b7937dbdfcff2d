"""Generates the golden fixtures of tests/golden/*.npz from the REFERENCE'S OWN
code (oracle/_ref/libpvref.so, built from the reference sources by
oracle/Makefile.ref).  Run in a checkout where the reference is present:

    python tests/golden/make_golden.py

Each fixture holds the input pattern/values/RHS of one seeded test matrix
(tests/matrices.py) and what the reference computes for it:
  perm_amd            AMD 1.1 ordering (004a_algorithm_amd_function.cpp:10-50)
  perm_rows ...       every symbolic array of prepare_matrices (000:10-93)
  csc_in              the scattered CSC values of one Newton iteration (000:193-210)
  lu_seq, lu_levels   GLU_CSC_CPU_sequential and the level-ordered CPU GLU
                      (GLU_CSC_CPU_levels_strings.cpp:65-132)
  x_perm              Substitute_LU_Vector_b_CSC_CPU on the permuted RHS with
                      lu_seq (GLU_CSC_CPU_Triangular.cpp:27-43)
  x                   the same solution in the caller's unknown order (000:233)

orderings/block_plant_amd.npz holds the reference's AMD ordering (and its
fill and level counts) of the reference-topology plants (plant.block_plant)
of 1 x 50 x 50 and 7 x 50 x 50 panels, too large for a full fixture: with the
ordering, the symbolic analysis reproduces the reference's arrays and the
oracle's restatement gives the reference's factors.  orderings/plant_amd.npz
holds the same for the benchmark's string/combiner plant (plant.Plant) of
50 x 24 x 28 panels.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import matrices as M  # noqa: E402
from oracle import oracle as O  # noqa: E402

FIXTURES = ("plant_1x2x2", "plant_c1", "mesh_12x10", "mesh_20x20", "random_300",
            "block_1x20x20")
BLOCK_ORDERINGS = ((1, 50, 50), (7, 50, 50))
PLANT_ORDERINGS = ((50, 24, 28),)


def fixtures() -> None:
    for name in FIXTURES:
        rp, ci, a, b = M.CASES[name]()
        ref = O.Ref(rp, ci)
        arrs = ref.arrays()
        n = len(rp) - 1
        csc = ref.scatter(a)
        lu_seq = ref.refactor(csc, sequential=True)
        lu_lev = ref.refactor(csc, sequential=False)
        p, q = arrs["perm_amd"], arrs["perm_rows"]
        t = np.empty(n)
        t[np.argsort(p)] = b          # apply_permutation(Pinv), util.cpp:61-68
        w = np.empty(n)
        w[q] = t                      # apply_permutation(Q)
        x_perm = ref.solve(lu_seq, w)
        x = np.empty(n)
        x[p] = x_perm                 # apply_permutation(P), 000:233
        np.savez_compressed(HERE / f"{name}.npz", rowptr=rp, colidx=ci, a=a, b=b, csc_in=csc,
                            lu_seq=lu_seq, lu_levels=lu_lev, x_perm=x_perm, x=x, **arrs)
        print(f"{name}: n={n} nnz_lu={len(csc)}")


def orderings(kind: str) -> None:
    """The reference's AMD ordering with its fill and level counts:
    kind "block" for plant.block_plant, "plant" for plant.Plant."""
    from phdthesis_albertojimenezruiz_gb300 import Plant

    out = {}
    for dims in (BLOCK_ORDERINGS if kind == "block" else PLANT_ORDERINGS):
        if kind == "block":
            rp, ci, _, _ = M.block(dims)
        else:
            p = Plant(*dims)
            rp, ci = p.rowptr, p.colidx
        ref = O.Ref(rp, ci)
        tag = "x".join(map(str, dims))
        out[f"perm_{tag}"] = ref.get("perm_amd")
        out[f"nnz_lu_{tag}"] = np.array(len(ref.get("csc_row")))
        out[f"u_levels_{tag}"] = np.array(len(ref.get("u_sl")) - 1)
        out[f"lu_levels_{tag}"] = np.array(len(ref.get("lu_sl")) - 1)
        print(f"{kind} {tag}: n={len(rp) - 1} nnz_lu={int(out[f'nnz_lu_{tag}'])} "
              f"u_levels={int(out[f'u_levels_{tag}'])}")
    (HERE / "orderings").mkdir(exist_ok=True)
    name = "block_plant_amd.npz" if kind == "block" else "plant_amd.npz"
    np.savez_compressed(HERE / "orderings" / name, **out)


def main() -> None:
    """Arguments select what to regenerate (fixtures, block, plant); none: all."""
    if O.build_ref() is None:
        raise SystemExit("reference sources not found; fixtures cannot be regenerated here")
    what = sys.argv[1:] or ["fixtures", "block", "plant"]
    if "fixtures" in what:
        fixtures()
    for kind in ("block", "plant"):
        if kind in what:
            orderings(kind)


if __name__ == "__main__":
    main()
