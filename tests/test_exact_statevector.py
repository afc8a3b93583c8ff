"""The annealing algorithm against the physics it emulates: an exact state-vector simulation of
the same Trotter circuit (oracle/exact_statevector.py, a restatement of the reference's exact
simulator, src/bqa/exact_sim.py:36-86).  On a tree, BP and the BP-gauged simple update are
exact while no bond is cut, so with a negligible pinv_eps the tensor-network results must
equal the state vector's (measured 4e-9 and 2e-7 on the two trees, held to 1e-6); the default
pinv_eps = 1e-6 cut costs ~5e-4.

The CPU test checks the oracle (and so the reference algorithm it restates); the GPU tests
check the CUDA path through bqa_gb300's own job API in both precisions."""
import logging

import numpy as np
import pytest

from bqa_gb300 import instances
from oracle import bqa_oracle as orc
from oracle.exact_statevector import StateVector, run_exact


def tree_job(n=10, seed=3, pinv_eps=1e-12, steps=12):
    rng = np.random.default_rng(seed)
    edges = np.array([(int(rng.integers(0, v)), v) for v in range(1, n)])
    return instances.qubo_config(edges, rng.normal(size=len(edges)), rng.normal(size=n), max_bond_dim=32,
                                 bp_eps=1e-12, pinv_eps=pinv_eps, max_bp_iter_number=200,
                                 schedule=instances.anneal_schedule(3.0, steps))


def test_state_vector_basics():
    st = StateVector(3)
    st.apply1(1, np.array([[0, 1], [1, 0]], dtype=complex))
    assert np.isclose(st.dens1(1)[1, 1], 1.0) and np.isclose(st.dens1(0)[0, 0], 1.0)
    st.apply_zz(0, 1, 0.3)   # diagonal: populations unchanged
    assert np.isclose(np.abs(st.psi).max(), 1.0)


@pytest.mark.parametrize("seed", [3, 7])
def test_oracle_anneal_equals_state_vector_on_a_tree(seed):
    logging.disable(logging.WARNING)
    conf = tree_job(seed=seed)
    exact = np.array(run_exact(conf)[0][1])
    tn = np.array(orc.run_qa(conf)[0][1])
    logging.disable(logging.NOTSET)
    assert np.abs(tn - exact).max() < 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize("precision,pinv_eps,tol", [("double", 1e-12, 1e-6), ("single", 1e-6, 2e-3)])
def test_gpu_anneal_equals_state_vector_on_a_tree(precision, pinv_eps, tol):
    from bqa_gb300.engine import Annealer
    from bqa_gb300.layout import build_context
    conf = tree_job(pinv_eps=pinv_eps)
    exact = np.array(run_exact(conf)[0][1])
    ctx = build_context(conf)
    job = Annealer(ctx, precision=precision)
    for ins in ctx.instructions:
        if isinstance(ins, dict):
            job.run_layer(ins["xtime"], ins["ztime"])
    got = job.bloch_vectors()
    err = np.abs(got - exact).max()
    print(f"{precision}: max Bloch error vs the exact state vector {err:.2e}")
    assert err < tol
