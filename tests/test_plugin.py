"""The gb300 backend inside the reference bqa package.

Without the reference (every host): contexts that bqa's own ``config_to_context`` built for
gb300 configs, recorded by tests/golden/make_plugin_context.py, convert into the engine's
context with maps bit-identical to the engine's own compiler.

With the reference (BQA_REFERENCE_SRC names its ``src`` directory; skipped otherwise): the
registered backend is a real ``Tensor`` subclass, bqa's config validation accepts "gb300",
``config_to_context`` runs unchanged on it, the converted context equals the engine's own, the
per-operation methods refuse, and ``bqa.run_qa`` hands gb300 contexts to
``plugin.run_context`` while other backends stay on the original path.
"""
import os
import sys
import tempfile
from pathlib import Path

import numpy as np
import pytest

from bqa_gb300 import plugin
from bqa_gb300.layout import build_context
from tests import golden_cases as gc

REF_SRC = Path(os.environ.get("BQA_REFERENCE_SRC", "")) if os.environ.get("BQA_REFERENCE_SRC") else None
GOLDEN = Path(__file__).resolve().parent / "golden"
RECORDED = ["mixed_n18_chi3", "rr3_n12_measure"]


def assert_same_context(got, want):
    assert (got.nodes_number, got.edges_number) == (want.nodes_number, want.edges_number)
    for k in ("max_bond_dim", "max_bp_iters_number", "bp_eps", "pinv_eps", "measurement_threshold", "damping",
              "seed"):
        assert getattr(got, k) == getattr(want, k), k
    assert list(got.degree_to_layout) == list(want.degree_to_layout)
    for d, L in want.degree_to_layout.items():
        G = got.degree_to_layout[d]
        for k in ("node_ids", "input_msgs_position", "output_msgs_position", "lmbds_position"):
            assert np.array_equal(getattr(G, k), getattr(L, k)), (d, k)
        assert np.array_equal(G.node_ampls, L.node_ampls) and np.array_equal(G.edge_ampls, L.edge_ampls)
    for k in ("node_degree", "node_position", "edge_src", "edge_dst", "edge_ampl", "node_ampl"):
        assert np.array_equal(getattr(got, k), getattr(want, k)), k
    steps = lambda ins: [(i["xtime"], i["ztime"]) if isinstance(i, dict) else i for i in ins]
    assert steps(got.instructions) == steps(want.instructions)


@pytest.mark.parametrize("name", RECORDED)
def test_recorded_reference_context_converts_bit_exactly(name):
    with np.load(GOLDEN / f"plugin_ctx_{name}.npz") as f:
        ref_ctx = plugin.reference_like_context({k: f[k] for k in f.files})
    assert_same_context(plugin.context_from_reference(ref_ctx), build_context(gc.config(name)))


@pytest.fixture(scope="module")
def bqa_mod():
    if REF_SRC is None or not (REF_SRC / "bqa").is_dir():
        pytest.skip("BQA_REFERENCE_SRC does not name the reference bqa sources")
    shim = Path(tempfile.mkdtemp(prefix="bqa_shim_"))
    (shim / "bqa-0.1.6.dist-info").mkdir()
    (shim / "bqa-0.1.6.dist-info" / "METADATA").write_text("Metadata-Version: 2.1\nName: bqa\nVersion: 0.1.6\n")
    os.environ.setdefault("BQA_PRECISION", "double")
    sys.path[:0] = [str(shim), str(REF_SRC)]
    import bqa
    assert plugin.register()
    assert plugin.register()   # idempotent
    return bqa


@pytest.mark.parametrize("name", ["tree9", "rr3_n16_chi4", "mixed_n18_chi3", "grid3x4_chi4_damped",
                                  "rr3_n12_measure"])
def test_reference_config_to_context_runs_on_the_gb300_backend(bqa_mod, name):
    from bqa.backends import BACKEND_STR_TO_BACKEND, Tensor
    from bqa.config.core import config_to_context
    cls = BACKEND_STR_TO_BACKEND["gb300"]
    assert issubclass(cls, Tensor) and not getattr(cls, "__abstractmethods__", None)
    ctx = config_to_context(gc.config(name, backend="gb300"))
    assert ctx.backend is cls
    assert_same_context(plugin.context_from_reference(ctx), build_context(gc.config(name)))
    # the recorder round-trips what the GPU test replays
    again = plugin.reference_like_context(plugin.record_context(ctx))
    assert_same_context(plugin.context_from_reference(again), build_context(gc.config(name)))


def test_per_operation_methods_refuse(bqa_mod):
    from bqa.backends import BACKEND_STR_TO_BACKEND
    cls = BACKEND_STR_TO_BACKEND["gb300"]
    t = cls.make_from_list([1, 2, 3])
    assert t.numpy.dtype == np.intp and t.raw_shape == ()
    with pytest.raises(NotImplementedError, match="fused"):
        cls.batched_matmul(t.raw_tensor, t.raw_tensor)


def test_run_qa_dispatches_gb300_contexts(bqa_mod, monkeypatch):
    from bqa.config.config_syntax import _analyse_config
    cfg = {"edges": {(0, 1): 1.0, (1, 2): -0.5}, "backend": "gb300",
           "schedule": {"total_time": 1.0, "actions": [{"weight": 1.0, "steps_number": 2}, "get_bloch_vectors"]}}
    assert _analyse_config(dict(cfg))["backend"] == "gb300"
    seen = []
    monkeypatch.setattr(plugin, "run_context", lambda ctx: seen.append(ctx) or [["bloch_vectors", []]])
    assert bqa_mod.run_qa(dict(cfg)) == [["bloch_vectors", []]]
    assert len(seen) == 1 and seen[0].backend.__name__ == "GB300Backend" and seen[0].nodes_number == 3
    out = bqa_mod.run_qa(dict(cfg, backend="numpy"))
    assert out[0][0] == "bloch_vectors" and len(out[0][1]) == 3
    assert len(seen) == 1
