"""Exact state-vector simulation of the annealing circuit -- TEST INFRASTRUCTURE ONLY.

A numpy restatement of the reference's exact simulator (``src/bqa/exact_sim.py:36-86``), whose
own state-vector backend (the Rust package ``qem``, git 8156bfd, not vendored) is absent: the
same initial product state (FLIPPED_HADAMARD on |0> of every qubit), the same per-step gate
order (Z gates exp(-i h t Z) on every node, ZZ gates exp(-i J t ZZ) on every undirected edge,
X gates exp(-i x X) on every node) and the same Bloch-vector read-out.  For up to ~16 qubits.

On a tree, BP and the BP-gauged simple update of the tensor-network algorithm are exact as
long as no bond is truncated, so the tensor-network annealer must reproduce this simulation
there up to the ``pinv_eps`` cut -- a check of the whole algorithm against the physics it
emulates, independent of the reference's implementation.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))

from bqa_gb300 import config as cfg  # noqa: E402

# src/bqa/exact_sim.py:14-30
FLIPPED_HADAMARD = np.array([[1.0, 1.0], [-1.0, 1.0]], dtype=np.complex128) / np.sqrt(2.0)
Z = np.diag([1.0, -1.0]).astype(np.complex128)
X = np.array([[0.0, 1.0], [1.0, 0.0]], dtype=np.complex128)
ZZ_DIAG = np.array([1.0, -1.0, -1.0, 1.0], dtype=np.complex128)


class StateVector:
    """n-qubit state as an array of shape (2,)*n, qubit q on axis q."""

    def __init__(self, n: int):
        self.n = n
        self.psi = np.zeros((2,) * n, dtype=np.complex128)
        self.psi[(0,) * n] = 1.0

    def apply1(self, q: int, u: np.ndarray) -> None:
        self.psi = np.moveaxis(np.tensordot(u, self.psi, axes=([1], [q])), 0, q)

    def apply_zz(self, a: int, b: int, t: float) -> None:
        # exp(-i t ZZ) = cos t I - i sin t ZZ, diagonal in the computational basis
        d = (np.cos(t) - 1j * np.sin(t) * ZZ_DIAG).reshape(2, 2)
        shape = [1] * self.n
        shape[a], shape[b] = 2, 2
        self.psi = self.psi * (d if a < b else d.T).reshape(shape)

    def dens1(self, q: int) -> np.ndarray:
        m = np.moveaxis(self.psi, q, 0).reshape(2, -1)
        return m @ m.conj().T


def _gate(t: float, p: np.ndarray) -> np.ndarray:
    return np.cos(t) * np.eye(2, dtype=np.complex128) - 1j * np.sin(t) * p


def bloch(rho: np.ndarray) -> np.ndarray:
    """[x, y, z] of a 2x2 density matrix (src/bqa/utils.py:23-27)."""
    return np.array([(rho[0, 1] + rho[1, 0]).real, (rho[1, 0] - rho[0, 1]).imag, (rho[0, 0] - rho[1, 1]).real])


def run_exact(config: dict) -> list:
    """``run_qa``-style result list of the exact simulation (Bloch vectors only; a
    measurement instruction is not reproducible in the reference either)."""
    c = cfg.analyse_config(dict(config))
    edges = c[cfg.EDGES_KEY]
    n = 1 + max(max(c[cfg.NODES_KEY].keys(), default=-1), max(max(a, b) for a, b in edges.keys()))
    fields = {v: c[cfg.NODES_KEY].get(v, c[cfg.DEFAULT_FIELD_KEY]) for v in range(n)}
    st = StateVector(n)
    for q in range(n):
        st.apply1(q, FLIPPED_HADAMARD)
    out = []
    seen = set()
    pairs = []
    for (a, b), j in edges.items():
        if (b, a) not in seen:
            seen.add((a, b))
            pairs.append((a, b, j))
    for ins in cfg.canonicalize_schedule(c[cfg.SCHEDULE_KEY]):
        if isinstance(ins, dict):
            for q in range(n):
                st.apply1(q, _gate(ins["ztime"] * fields[q], Z))
            for a, b, j in pairs:
                st.apply_zz(a, b, ins["ztime"] * j)
            for q in range(n):
                st.apply1(q, _gate(ins["xtime"], X))
        elif ins == cfg.GET_BLOCH_VECTORS:
            out.append(["bloch_vectors", [bloch(st.dens1(q)).tolist() for q in range(n)]])
    return out
