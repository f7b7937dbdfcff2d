"""The benchmark's two host-buffer workloads describe the same Jacobians
(CPU): the panel conductances of make_conductances, stamped into the plant's
linear part, give make_inputs' A values."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
import bench  # noqa: E402


def test_conductances_reproduce_assembled_values():
    S, ld = 3, 64
    p, a, _ = bench.make_inputs(S, ld, seed0=1000)
    g = bench.make_conductances(p, S, ld, seed0=1000)
    assert g.shape == (p.n_panels, ld) and not g[:, S:].any()
    for s in range(S):
        a_s = p.jacobian_values(g[:, s])
        assert np.allclose(a_s, a[:, s], rtol=1e-14, atol=0.0)
