"""pvglu_solve_noalloc: the solve whose work vector lives in the library's
static device array, for callers whose solve path must not allocate device
memory (an application that reserves the GPU's memory up front, or a loop
that cannot take an allocation's implicit synchronisation).  Checked through
the C ABI against the ordinary pvglu_solve on two calls in a row (the array
keeps the previous call's contents) and against the CPU oracle, in every
schedule, single and batched (the batched chain programs move the static
array's rows with bulk copies), and for its size limit.  Kept in a file of
its own that pytest collects last.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest
from conftest import norm_err

from oracle import oracle as O
from phdthesis_albertojimenezruiz_gb300 import (FP64, SCHED_LEVELS, SCHED_PERSISTENT,
                                                SCHED_THREAD_CHAIN, Numeric, Plant, Symbolic)
from phdthesis_albertojimenezruiz_gb300 import _native as N

pytestmark = pytest.mark.gpu
TOL64 = 1e-12  # the tolerance of the FP64 parity tests


def _noalloc(num: Numeric, x, flags: int) -> int:
    return N.lib().pvglu_solve_noalloc(num.handle, C.c_void_p(x.data_ptr()), flags,
                                       C.c_void_p(0))


@pytest.mark.parametrize("schedule", [SCHED_LEVELS, SCHED_PERSISTENT, SCHED_THREAD_CHAIN])
@pytest.mark.parametrize("S", [1, 8, 64])
def test_noalloc_matches_solve_twice(cuda, schedule, S):
    import torch

    import matrices as M

    p = Plant(10, 16, 20)
    s = Symbolic(p.rowptr, p.colidx)
    o = O.Port(p.rowptr, p.colidx, s.array("perm_amd"))
    num = Numeric(s, S, FP64, schedule)
    a, _ = M.plant_batch(p, S, seed0=41)
    a_pad = np.zeros((a.shape[0], num.ld))
    a_pad[:, :S] = a
    num.scatter(torch.from_numpy(a_pad).cuda())
    num.refactor()
    assert num.check()[0] == 0
    rng = np.random.default_rng(3)
    for call, flags in enumerate((N.SOLVE_ORIGINAL, N.SOLVE_ORIGINAL | N.SOLVE_TRANSPOSE)):
        b = np.zeros((s.n, num.ld))
        b[:, :S] = rng.uniform(-1, 1, (s.n, S))
        want = torch.from_numpy(b).cuda()
        num.solve(want, transpose=bool(flags & N.SOLVE_TRANSPOSE), original=True)
        got = torch.from_numpy(b).cuda()
        N.check(_noalloc(num, got, flags), f"pvglu_solve_noalloc call {call + 1}")
        torch.cuda.synchronize()
        w, g = want.cpu().numpy()[:, :S], got.cpu().numpy()[:, :S]
        for k in range(S):
            assert norm_err(g[:, k], w[:, k]) <= TOL64, (call, k)
        if not flags & N.SOLVE_TRANSPOSE:
            for k in sorted({0, S // 2, S - 1}):
                _, x_ref = o.scatter_refactor_solve(a[:, k], b[:, k])
                assert norm_err(g[:, k], x_ref) <= TOL64, (call, k)


def test_noalloc_rejects_oversized_handle(cuda):
    import torch

    p = Plant(50, 24, 28)  # 33,750 unknowns x 64 scenarios > 1,048,576 entries
    s = Symbolic(p.rowptr, p.colidx)
    num = Numeric(s, 64, FP64, SCHED_LEVELS)
    x = torch.zeros(s.n * num.ld, dtype=torch.float64, device="cuda")
    rc = _noalloc(num, x, N.SOLVE_ORIGINAL)
    assert rc == 9  # PVGLU_ERR_TOO_LARGE
    assert b"exceeds the static scratch" in N.lib().pvglu_last_error()
