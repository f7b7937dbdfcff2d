"""Seeded test matrices (patterns + values) for the parity tests.

* plant(dims): the synthetic PV plant's companion Jacobian at the flat start
  with seeded shadows (tree-structured MNA, voltage-source rows with zero
  diagonals);
* mesh(nx, ny): a 2-D resistor grid with voltage sources on some nodes (fill,
  long dependency chains, merged chain levels);
* random_mna(n): random unsymmetric sparse conductance pattern plus
  voltage-source rows/columns (structurally zero diagonals, row exchanges).

Values are diagonally dominant on the node rows so that the pivot-free LU
is stable, as for the circuit matrices the reference factors.
"""
from __future__ import annotations

import numpy as np


def _csr_from_dict(n, entries):
    rows = [[] for _ in range(n)]
    for (i, j), v in entries.items():
        rows[i].append((j, v))
    rowptr = [0]
    col, val = [], []
    for r in rows:
        r.sort()
        col += [c for c, _ in r]
        val += [v for _, v in r]
        rowptr.append(len(col))
    return (np.array(rowptr, np.int32), np.array(col, np.int32), np.array(val, np.float64))


def _stamp(entries, i, j, g):
    def add(a, b, v):
        if a >= 0 and b >= 0:
            entries[(a, b)] = entries.get((a, b), 0.0) + v
    add(i, i, g)
    add(i, j, -g)
    add(j, i, -g)
    add(j, j, g)


def _source(entries, node, row, rhs, vs):
    entries[(node, row)] = entries.get((node, row), 0.0) - 1.0
    entries[(row, node)] = entries.get((row, node), 0.0) + 1.0
    rhs[row] = vs


def mesh(nx: int, ny: int, n_sources: int = 3, seed: int = 0):
    rng = np.random.default_rng(seed)
    nn = nx * ny
    n = nn + n_sources
    e = {}
    rhs = np.zeros(n)
    idx = lambda x, y: y * nx + x  # noqa: E731
    for y in range(ny):
        for x in range(nx):
            if x + 1 < nx:
                _stamp(e, idx(x, y), idx(x + 1, y), rng.uniform(1, 10))
            if y + 1 < ny:
                _stamp(e, idx(x, y), idx(x, y + 1), rng.uniform(1, 10))
            _stamp(e, idx(x, y), -1, rng.uniform(0.01, 0.1))  # leak to ground
    nodes = rng.choice(nn, size=n_sources, replace=False)
    for k, nd in enumerate(nodes):
        _source(e, int(nd), nn + k, rhs, rng.uniform(10, 100))
    rhs[:nn] = rng.uniform(-1, 1, nn)
    rp, ci, v = _csr_from_dict(n, e)
    return rp, ci, v, rhs


def random_mna(n_nodes: int, avg_deg: float = 3.0, n_sources: int = 4, seed: int = 0):
    """Random unsymmetric conductance-like pattern + voltage sources."""
    rng = np.random.default_rng(seed)
    n = n_nodes + n_sources
    e = {}
    rhs = np.zeros(n)
    m = int(n_nodes * avg_deg / 2)
    for _ in range(m):
        i, j = rng.integers(0, n_nodes, 2)
        if i == j:
            continue
        _stamp(e, int(i), int(j), rng.uniform(0.5, 5))
    # unsymmetric couplings (controlled sources): one-sided entries
    for _ in range(n_nodes // 4):
        i, j = rng.integers(0, n_nodes, 2)
        if i != j:
            e[(int(i), int(j))] = e.get((int(i), int(j)), 0.0) + rng.uniform(-0.2, 0.2)
    for i in range(n_nodes):
        e[(i, i)] = e.get((i, i), 0.0) + rng.uniform(1, 2)
        # make strictly diagonally dominant by rows
        off = sum(abs(v) for (a, b), v in e.items() if a == i and b != i)
        e[(i, i)] += off
    nodes = rng.choice(n_nodes, size=n_sources, replace=False)
    for k, nd in enumerate(nodes):
        _source(e, int(nd), n_nodes + k, rhs, rng.uniform(1, 10))
    rhs[:n_nodes] = rng.uniform(-1, 1, n_nodes)
    rp, ci, v = _csr_from_dict(n, e)
    return rp, ci, v, rhs


def plant(dims, seed: int = 1, preset: str = "c1"):
    """(rowptr, colidx, A values, b) of the plant's companion system."""
    from phdthesis_albertojimenezruiz_gb300 import Plant

    p = Plant(*dims)
    g = p.irradiance(seed=seed, preset=preset)
    _, _, a, b = p.companion(g, p.flat_start())
    return p.rowptr.copy(), p.colidx.copy(), a, b


def plant_batch(p, n_scenarios: int, seed0: int = 1, preset: str = "c1", t: float = 0.0):
    """A values [nnz_a, S] and b [n, S] for S seeded shadow fields."""
    a = np.empty((len(p.a_lin), n_scenarios))
    b = np.empty((p.n, n_scenarios))
    v = p.flat_start()
    for s in range(n_scenarios):
        g = p.irradiance(seed=seed0 + s, t=t, preset=preset)
        _, _, a[:, s], b[:, s] = p.companion(g, v)
    return a, b


def block(dims, seed: int = 0):
    """(rowptr, colidx, A values, b) of a plant with the reference's own
    topology (plant.block_plant): dense bus rows and columns after fill."""
    from phdthesis_albertojimenezruiz_gb300.plant import block_plant

    return block_plant(*dims, seed=seed)


CASES = {
    "plant_1x2x2": lambda: plant((1, 2, 2)),
    "plant_c1": lambda: plant((4, 8, 20)),
    "mesh_12x10": lambda: mesh(12, 10, 3, seed=3),
    "mesh_20x20": lambda: mesh(20, 20, 4, seed=4),
    "mesh_30x30": lambda: mesh(30, 30, 5, seed=4),
    "random_300": lambda: random_mna(300, 3.0, 6, seed=5),
    "random_1500": lambda: random_mna(1500, 2.5, 10, seed=6),
    "block_1x20x20": lambda: block((1, 20, 20), seed=8),
}
