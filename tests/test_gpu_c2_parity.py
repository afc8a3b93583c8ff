"""Parity at the headline shape: a 10,000-node instance of the 100k-qubit workload's generator
(random 3-regular, J = +-1, h ~ U(-0.5, 0.5), chi 16), first 66 steps of the 200-step schedule
(past bond-dim saturation), against the REFERENCE run at FP64 (fixture written by
tests/golden/make_golden_c2.py).  complex128 to round-off (measured 2.4e-13); complex64
measured at 1.2e-4, held to 1.5x that."""
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

import bqa_gb300  # noqa: E402
from tests.golden.make_golden_c2 import config_from_fixture  # noqa: E402

FIXTURE = Path(__file__).resolve().parent / "golden" / "c2_rr3_n10k_chi16.npz"


@pytest.fixture(scope="module")
def case():
    if not FIXTURE.exists():
        pytest.skip("fixture not generated")
    return config_from_fixture(FIXTURE), np.load(FIXTURE)["bloch"]


def _bloch(conf, precision, monkeypatch):
    monkeypatch.setenv("BQA_PRECISION", precision)
    out = bqa_gb300.run_qa(dict(conf), as_arrays=True)
    return out[0][1]


def test_complex128_matches_reference(case, monkeypatch):
    conf, want = case
    got = _bloch(conf, "double", monkeypatch)
    assert got.shape == want.shape
    err = np.abs(got - want).max()
    print(f"complex128 vs reference: max Bloch error {err:.3e}")
    assert err < 1e-8


def test_complex64_within_bar(case, monkeypatch):
    """Measured 1.21e-4 max (4.5e-6 mean on <Z>); held to 1.8e-4."""
    conf, want = case
    got = _bloch(conf, "single", monkeypatch)
    err = np.abs(got - want).max()
    print(f"complex64 vs reference: max Bloch error {err:.3e}, mean |<Z> error| "
          f"{np.abs(got[:, 2] - want[:, 2]).mean():.3e}")
    assert err < 1.8e-4, err


def test_complex64_mixed_precision_within_bar(case, monkeypatch):
    """Mixed-precision BP (BF16 tensor-core sweeps while the BP distance is above 2^-5, FP32
    sweeps to the tolerance): held to the 1e-3 <Z> bar stated for the mixed-precision form."""
    conf, want = case
    monkeypatch.setenv("BQA_GB300_MIXED", "1")
    got = _bloch(conf, "single", monkeypatch)
    err = np.abs(got - want).max()
    print(f"complex64 mixed vs reference: max Bloch error {err:.3e}, mean |<Z> error| "
          f"{np.abs(got[:, 2] - want[:, 2]).mean():.3e}")
    assert err < 1e-3, err


_CUDA_CORE_SCRIPT = """
import sys, numpy as np, bqa_gb300
from tests.test_gpu_c2_parity import FIXTURE
from tests.golden.make_golden_c2 import config_from_fixture
conf, want = config_from_fixture(FIXTURE), np.load(FIXTURE)["bloch"]
got = bqa_gb300.run_qa(dict(conf), as_arrays=True)[0][1]
err = float(np.abs(got - want).max())
print(f"complex64 on the CUDA-core message kernel vs reference: max Bloch error {err:.3e}")
sys.exit(0 if err < 1.8e-4 else 3)
"""


def test_complex64_cuda_core_kernel_within_bar(case):
    """BQA_GB300_TC=0 at load: the degree-3 bond-dim-16 sweeps on the CUDA-core kernel instead of
    the 2xFP16 tensor-core default, held to the same bar."""
    import os
    import subprocess
    import sys
    root = Path(__file__).resolve().parents[1]
    env = dict(os.environ, BQA_GB300_TC="0", BQA_PRECISION="single", PYTHONPATH=str(root))
    r = subprocess.run([sys.executable, "-c", _CUDA_CORE_SCRIPT], cwd=root, env=env, timeout=900)
    assert r.returncode == 0
