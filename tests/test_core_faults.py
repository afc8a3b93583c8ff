"""Host logic of the tensor-core fault check in ``core.run_compiled`` (no GPU: the job is a
fake whose library reports a chosen fault count)."""
import types

import numpy as np
import pytest

from bqa_gb300 import config as cfg
from bqa_gb300 import core


class _FakeLib:
    def __init__(self, faults):
        self.faults = faults
        self.reads = 0

    def tc_faults(self, stream=None, reset=True):
        self.reads += 1
        return self.faults


def _fake_annealer(faults, jobs):
    class FakeJob:
        def __init__(self, ctx, device=None):
            self.lib = _FakeLib(faults)
            self.stream = 0
            self.layers = 0
            jobs.append(self)

        def run_layer(self, xtime, ztime):
            self.layers += 1

        def bloch_vectors(self):
            return np.zeros((2, 3))

    return FakeJob


CTX = types.SimpleNamespace(instructions=[{"xtime": 0.1, "ztime": 0.2}, cfg.GET_BLOCH_VECTORS])


def test_healthy_job_returns_its_results(monkeypatch):
    jobs = []
    monkeypatch.setattr(core, "Annealer", _fake_annealer(0, jobs))
    out = core.run_compiled(CTX)
    assert out == [["bloch_vectors", [[0.0, 0.0, 0.0], [0.0, 0.0, 0.0]]]]
    assert jobs[0].layers == 1 and jobs[0].lib.reads == 1


def test_tensor_core_timeout_voids_the_job(monkeypatch):
    jobs = []
    monkeypatch.setattr(core, "Annealer", _fake_annealer(2, jobs))
    with pytest.raises(RuntimeError, match="2 tensor-core CTA"):
        core.run_compiled(CTX)
    assert jobs[0].lib.reads == 1
