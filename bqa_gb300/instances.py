"""Seeded QUBO instance generators for annealing jobs (numpy only, no networkx).

The reference builds its benchmark instances with networkx (``src/bqa/benchmarking.py:51-72``:
``generate_qubo_on_random_regular_graph``, ``generate_qubo_on_2d_grid``).  These generators
produce the same graph families and return the same ``(nodes, edges)`` dicts, so their
output drops into a job config; they are written for 10^5-10^6 nodes (vectorised stub
matching) and need nothing beyond numpy.  Graphs are not bit-identical to networkx's
(different sampling algorithm); every test that compares against the reference stores its
edge list.

Random d-regular graphs: configuration model (uniform random matching of d stubs per
node), then self-loops and repeated edges are removed by random double-edge swaps that
keep every degree, which is the standard repair of the pairing model.
"""
from __future__ import annotations

import numpy as np


def _repair(edges: np.ndarray, rng: np.random.Generator, max_rounds: int = 10000) -> np.ndarray:
    """Remove self-loops and multi-edges by degree-preserving double-edge swaps."""
    edges = edges.copy()
    m = edges.shape[0]
    for _ in range(max_rounds):
        a, b = edges[:, 0], edges[:, 1]
        lo, hi = np.minimum(a, b), np.maximum(a, b)
        key = lo.astype(np.int64) * (int(edges.max()) + 1) + hi
        order = np.argsort(key, kind="stable")
        dup = np.zeros(m, dtype=bool)
        dup[order[1:]] = key[order[1:]] == key[order[:-1]]
        bad = np.flatnonzero((a == b) | dup)
        if bad.size == 0:
            return edges
        for i in bad:
            j = int(rng.integers(m))
            if j == i:
                continue
            u, v = edges[i]
            x, y = edges[j]
            if rng.integers(2):
                x, y = y, x
            # (u,v),(x,y) -> (u,x),(v,y)
            if u == x or v == y:
                continue
            edges[i] = (u, x)
            edges[j] = (v, y)
    raise RuntimeError("could not make the random graph simple")


def random_regular_edges(n: int, d: int, seed: int) -> np.ndarray:
    """(n*d/2, 2) edge array of a simple random d-regular graph on n nodes."""
    if (n * d) % 2 or d >= n:
        raise ValueError("n*d must be even and d < n")
    rng = np.random.default_rng(seed)
    stubs = np.repeat(np.arange(n, dtype=np.int64), d)
    rng.shuffle(stubs)
    edges = stubs.reshape(-1, 2)
    return _repair(edges, rng)


def configuration_model_edges(degrees: np.ndarray, seed: int) -> np.ndarray:
    """Simple graph with the given degree sequence (sum must be even)."""
    degrees = np.asarray(degrees, dtype=np.int64)
    if degrees.sum() % 2:
        raise ValueError("degree sum must be even")
    rng = np.random.default_rng(seed)
    stubs = np.repeat(np.arange(degrees.size, dtype=np.int64), degrees)
    rng.shuffle(stubs)
    return _repair(stubs.reshape(-1, 2), rng)


def periodic_grid_edges(rows: int, cols: int) -> np.ndarray:
    """Edges of the rows x cols torus (every node degree 4 for rows, cols >= 3)."""
    idx = np.arange(rows * cols, dtype=np.int64).reshape(rows, cols)
    right = np.stack([idx.ravel(), np.roll(idx, -1, axis=1).ravel()], axis=1)
    down = np.stack([idx.ravel(), np.roll(idx, -1, axis=0).ravel()], axis=1)
    return np.concatenate([right, down])


def qubo_config(edges: np.ndarray, couplings: np.ndarray, fields: np.ndarray, **params) -> dict:
    """Job config dict (reference DSL) from an edge array and amplitudes."""
    cfg = {
        "nodes": {int(v): float(h) for v, h in enumerate(fields)},
        "edges": {(int(a), int(b)): float(J) for (a, b), J in zip(edges, couplings)},
    }
    cfg.update(params)
    return cfg


def anneal_schedule(total_time: float, steps: int, readout: str | None = "get_bloch_vectors") -> dict:
    actions = [{"weight": 1.0, "steps_number": steps, "final_mixing": 0.0}]
    if readout:
        actions.append(readout)
    return {"total_time": total_time, "starting_mixing": 1.0, "actions": actions}


def headline_cpu_job(n: int = 1000, seed: int = 0) -> dict:
    """Random 3-regular, J, h ~ N(0,1), chi 4, 100 steps, T 10, tol 1e-6, <= 100 sweeps."""
    rng = np.random.default_rng(seed)
    e = random_regular_edges(n, 3, seed)
    return qubo_config(e, rng.normal(size=len(e)), rng.normal(size=n), max_bond_dim=4, bp_eps=1e-6,
                       pinv_eps=1e-6, max_bp_iter_number=100, schedule=anneal_schedule(10.0, 100))


def headline_gpu_job(n: int = 100_000, seed: int = 0, chi: int = 16, steps: int = 200,
                     total_time: float = 20.0, degree: int = 3) -> dict:
    """Random 3-regular, J in {-1,+1}, h ~ U(-0.5, 0.5), chi 16, 200 steps, T 20, tol 1e-5,
    <= 50 sweeps (the 100k-qubit FP32 configuration); `degree` changes the regular degree."""
    rng = np.random.default_rng(seed)
    e = random_regular_edges(n, degree, seed)
    J = 2.0 * rng.integers(0, 2, size=len(e)) - 1.0
    h = rng.uniform(-0.5, 0.5, size=n)
    return qubo_config(e, J, h, max_bond_dim=chi, bp_eps=1e-5, pinv_eps=1e-6, max_bp_iter_number=50,
                       schedule=anneal_schedule(total_time, steps))


def mixed_degree_job(rows: int = 300, cols: int = 300, extra: int = 50_000, chi: int = 8, steps: int = 150,
                     seed: int = 0, total_time: float = 15.0) -> dict:
    """Periodic grid (degree 4) plus a configuration-model graph of `extra` nodes with degrees
    uniform in {2, 3, 5, 6}; J ~ N(0,1), h ~ N(0, 0.3)."""
    rng = np.random.default_rng(seed)
    g = periodic_grid_edges(rows, cols)
    deg = rng.choice(np.array([2, 3, 5, 6]), size=extra)
    if deg.sum() % 2:
        deg[0] = 3 if deg[0] != 3 else 2
    c = configuration_model_edges(deg, seed + 1) + rows * cols
    e = np.concatenate([g, c])
    n = rows * cols + extra
    return qubo_config(e, rng.normal(size=len(e)), rng.normal(0.0, 0.3, size=n), max_bond_dim=chi, bp_eps=1e-5,
                       pinv_eps=1e-6, max_bp_iter_number=50, schedule=anneal_schedule(total_time, steps))
