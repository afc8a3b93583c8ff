"""The backend registers into the reference bqa (skipped unless BQA_REFERENCE_SRC names the
reference's ``src`` directory): bqa's own validation accepts "gb300", and bqa.run_qa hands
such configs to bqa_gb300.run_qa while other backends stay on the original path."""
import os
import sys
import tempfile
from pathlib import Path

import pytest

REF_SRC = Path(os.environ.get("BQA_REFERENCE_SRC", "")) if os.environ.get("BQA_REFERENCE_SRC") else None


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
    return bqa


def test_register_and_dispatch(bqa_mod, monkeypatch):
    import bqa_gb300.core
    from bqa_gb300 import plugin
    assert plugin.register()
    assert plugin.register()   # idempotent
    from bqa.backends import BACKEND_STR_TO_BACKEND
    from bqa.config.config_syntax import _analyse_config
    assert "gb300" in BACKEND_STR_TO_BACKEND
    cfg = {"edges": {(0, 1): 1.0, (1, 2): -0.5}, "backend": "gb300",
           "schedule": {"total_time": 1.0, "actions": [{"weight": 1.0, "steps_number": 2}, "get_bloch_vectors"]}}
    assert _analyse_config(dict(cfg))["backend"] == "gb300"
    calls = []
    monkeypatch.setattr(bqa_gb300.core, "run_qa", lambda c: calls.append(c) or [["bloch_vectors", []]])
    assert bqa_mod.run_qa(dict(cfg)) == [["bloch_vectors", []]]
    assert calls and calls[0]["backend"] == "gb300"
    numpy_cfg = dict(cfg, backend="numpy")
    out = bqa_mod.run_qa(numpy_cfg)
    assert out[0][0] == "bloch_vectors" and len(out[0][1]) == 3
    assert len(calls) == 1
    with pytest.raises(NotImplementedError):
        BACKEND_STR_TO_BACKEND["gb300"].make_from_list([1, 2])
