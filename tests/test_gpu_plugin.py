"""bqa.run_qa's gb300 dispatch target on the GPU: contexts that the reference's own
config_to_context built for gb300 configs (recorded by tests/golden/make_plugin_context.py;
the GPU hosts cannot import bqa) run through bqa_gb300.plugin.run_context and reproduce the
reference's FP64 results: Bloch vectors to 1e-3 in complex64 and 1e-9 in complex128,
measurement outcomes identical."""
from pathlib import Path

import numpy as np
import pytest

from tests import golden_cases as gc

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from bqa_gb300 import plugin  # noqa: E402

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("name", ["mixed_n18_chi3", "rr3_n12_measure"])
@pytest.mark.parametrize("precision,tol", [("single", 1e-3), ("double", 1e-9)])
def test_run_context_reproduces_the_reference(name, precision, tol, monkeypatch):
    monkeypatch.setenv("BQA_PRECISION", precision)
    with np.load(GOLDEN / f"plugin_ctx_{name}.npz") as f:
        ref_ctx = plugin.reference_like_context({k: f[k] for k in f.files})
    out = plugin.run_context(ref_ctx, as_arrays=True)
    want = gc.arrays(name)
    kinds = gc.manifest()[name]["results"]
    assert [o[0] for o in out] == kinds
    for i, kind in enumerate(kinds):
        ref = want[f"result{i}_{kind}"]
        if kind == "bloch_vectors":
            err = float(np.abs(out[i][1] - ref).max())
            print(f"{name} {precision}: max Bloch error {err:.2e}")
            assert err < tol
        else:
            assert np.array_equal(out[i][1], ref)
