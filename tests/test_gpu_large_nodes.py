"""Degrees 5 and 6 at bond dim up to 8: node tensors far beyond shared memory run on the
global-memory kernels (work tensors in caller scratch).  A full anneal on such a graph against
the FP64 oracle: complex128 to round-off, complex64 within the complex64 bar."""
import numpy as np
import pytest

from bqa_gb300 import instances
from oracle import bqa_oracle as orc

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from bqa_gb300.engine import Annealer  # noqa: E402
from bqa_gb300.layout import build_context  # noqa: E402


def _config():
    rng = np.random.default_rng(3)
    degs = np.array([6, 6, 5, 5, 3, 3, 3, 3, 2, 2, 2, 2])
    e = instances.configuration_model_edges(degs, 11)
    return instances.qubo_config(e, rng.normal(size=len(e)), rng.normal(0, 0.3, size=degs.size), max_bond_dim=8,
                                 bp_eps=1e-8, pinv_eps=1e-6, max_bp_iter_number=60,
                                 schedule=instances.anneal_schedule(1.2, 12))


@pytest.fixture(scope="module")
def oracle_bloch():
    return np.array(orc.run_qa(_config())[0][1])


def _run(precision):
    ctx = build_context(_config())
    job = Annealer(ctx, precision=precision)
    assert job.scratch is not None          # the degree-5/6 classes need the global kernels
    for ins in ctx.instructions:
        if isinstance(ins, dict):
            job.run_layer(ins["xtime"], ins["ztime"])
    return job.bloch_vectors(), [s["bond_dim"] for s in job.stats]


def test_complex128_matches_oracle(oracle_bloch):
    bloch, dims = _run("double")
    assert max(dims) >= 5                   # degree 5 and 6 at bond dim >= 5 exceed shared memory
    assert np.abs(bloch - oracle_bloch).max() < 1e-8


def test_complex64_within_bar(oracle_bloch):
    bloch, _ = _run("single")
    assert np.abs(bloch - oracle_bloch).max() < 5e-3
