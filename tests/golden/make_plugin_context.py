"""Record contexts that the REFERENCE's own config compiler builds for the gb300 backend.

Run where the reference sources are available, with BQA_REFERENCE_SRC naming the
reference's ``src`` directory:

    BQA_REFERENCE_SRC=<reference checkout>/src python tests/golden/make_plugin_context.py

For a few golden cases it registers the gb300 backend into the reference (bqa_gb300.plugin),
runs bqa's ``config_to_context`` on the config with ``"backend": "gb300"`` and writes the
context's maps, amplitudes and instruction list as plain arrays to
``tests/golden/plugin_ctx_<case>.npz`` (bqa_gb300.plugin.record_context).  The GPU test
rebuilds the context from that file (the GPU hosts cannot import bqa) and runs it through
``bqa_gb300.plugin.run_context``, the function bqa.run_qa dispatches gb300 configs to.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from tests import golden_cases as gc  # noqa: E402
from tests.golden.make_golden import _import_reference  # noqa: E402

CASES = ["mixed_n18_chi3", "rr3_n12_measure"]


def main():
    _import_reference()
    from bqa.config.core import config_to_context
    from bqa_gb300 import plugin
    assert plugin.register()
    for name in CASES:
        ctx = config_to_context(gc.config(name, backend="gb300"))
        np.savez(HERE / f"plugin_ctx_{name}.npz", **plugin.record_context(ctx))
        print(f"wrote plugin_ctx_{name}.npz")


if __name__ == "__main__":
    main()
