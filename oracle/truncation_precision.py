"""How much of the complex64 path's error comes from the truncation factorisations?

Test infrastructure, not part of the backend: runs the numpy oracle (a restatement of the
reference algorithm) three times on the same job and compares Bloch vectors:

  * complex128 everywhere (the reference's FP64 result);
  * complex64 everywhere (the reference's BQA_PRECISION=single arithmetic);
  * complex64 with the truncation factorisations -- the SVDs of the extended messages and of
    the bond kernels, src/bqa/state.py:171-200 -- done in complex128 on the complex64 inputs,
    their outputs rounded back to complex64.

    python oracle/truncation_precision.py [n]      # default: the 1000-qubit chi-4 job (~70 s)

It prints the maximum and mean Bloch-vector error of the two complex64 runs against the
complex128 run.
"""
from __future__ import annotations

import logging
import sys
import time
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))

from bqa_gb300 import instances  # noqa: E402
from oracle import bqa_oracle as orc  # noqa: E402


def anneal(conf: dict, dtype, fp64_truncation: bool = False) -> np.ndarray:
    octx = orc.make_context(dict(conf), dtype=dtype)
    st = orc.initialize_state(octx)
    original = orc.get_canonicalizers
    if fp64_truncation:
        def canonicalizers(msgs, eps):
            lam, can = original(msgs.astype(np.complex128), eps)
            return lam.astype(msgs.real.dtype), can.astype(msgs.dtype)
        orc.get_canonicalizers = canonicalizers
    try:
        for ins in octx.instructions:
            if isinstance(ins, dict):
                orc.run_layer(octx, ins["xtime"], ins["ztime"], st)
    finally:
        orc.get_canonicalizers = original
    return orc.bloch_vectors(orc.get_density_matrices(octx, st))


def main() -> None:
    logging.disable(logging.WARNING)
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 1000
    conf = instances.headline_cpu_job(n=n)
    t0 = time.time()
    ref = anneal(conf, np.complex128)
    print(f"complex128: {time.time() - t0:.1f} s")
    for label, kw in (("complex64", {}), ("complex64 + complex128 truncation", {"fp64_truncation": True})):
        got = anneal(conf, np.complex64, **kw)
        err = np.abs(got - ref)
        print(f"{label}: max Bloch error {err.max():.3e}, mean {err.mean():.3e}")


if __name__ == "__main__":
    main()
