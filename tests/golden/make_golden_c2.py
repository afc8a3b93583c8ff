"""Golden fixture at the headline shape: the REFERENCE bqa (v0.1.6) numpy backend at FP64 on a
10,000-node instance of the 100k-qubit workload's generator (random 3-regular, J = +-1,
h ~ U(-0.5, 0.5), chi 16, bp_eps 1e-5, <= 50 sweeps), over the first 66 steps of its
200-step, T = 20 schedule -- past the step at which the bond dimension saturates at 16.

Run where the reference sources are available, with BQA_REFERENCE_SRC naming the
reference's ``src`` directory:

    BQA_REFERENCE_SRC=<reference checkout>/src python tests/golden/make_golden_c2.py

(about an hour of one CPU core).  It writes tests/golden/c2_rr3_n10k_chi16.npz with the
instance (edges, couplings, fields), the schedule parameters and the reference's Bloch
vectors.  The GPU test reads only that file.
"""
from __future__ import annotations

import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from tests.golden.make_golden import _import_reference  # noqa: E402

N, STEPS_FULL, T_FULL, STEPS = 10_000, 200, 20.0, 66


def c2_config():
    """The config of the fixture, built from the committed generator."""
    from bqa_gb300 import instances
    conf = instances.headline_gpu_job(n=N, seed=0, chi=16, steps=STEPS_FULL, total_time=T_FULL)
    # the first STEPS steps of the STEPS_FULL-step schedule: same dt and mixing ramp
    conf["schedule"] = {"total_time": T_FULL * STEPS / STEPS_FULL, "starting_mixing": 1.0,
                        "actions": [{"weight": 1.0, "steps_number": STEPS,
                                     "final_mixing": 1.0 - STEPS / STEPS_FULL}, "get_bloch_vectors"]}
    return conf


def config_from_fixture(path: Path) -> dict:
    f = np.load(path)
    edges = {(int(u), int(v)): float(j) for (u, v), j in zip(f["edges"], f["couplings"])}
    nodes = {i: float(h) for i, h in enumerate(f["fields"])}
    return {"edges": edges, "nodes": nodes, "max_bond_dim": int(f["chi"]), "bp_eps": float(f["bp_eps"]),
            "pinv_eps": float(f["pinv_eps"]), "max_bp_iter_number": int(f["max_bp_iter"]),
            "schedule": {"total_time": float(f["total_time"]), "starting_mixing": 1.0,
                         "actions": [{"weight": 1.0, "steps_number": int(f["steps"]),
                                      "final_mixing": float(f["final_mixing"])}, "get_bloch_vectors"]}}


def main():
    import logging
    logging.basicConfig(level=logging.INFO, format="%(asctime)s %(message)s")
    conf = c2_config()
    _, _, run_qa = _import_reference()
    t0 = time.time()
    out = run_qa(dict(conf, backend="numpy"))
    secs = time.time() - t0
    bloch = np.array(out[0][1], dtype=np.float64)
    edges = np.array(list(conf["edges"].keys()), dtype=np.int32)
    path = HERE / "c2_rr3_n10k_chi16.npz"
    np.savez_compressed(path, edges=edges, couplings=np.array(list(conf["edges"].values())),
                        fields=np.array([conf["nodes"][i] for i in range(N)]), chi=16,
                        bp_eps=conf["bp_eps"], pinv_eps=conf["pinv_eps"],
                        max_bp_iter=conf["max_bp_iter_number"], total_time=conf["schedule"]["total_time"],
                        steps=STEPS, final_mixing=1.0 - STEPS / STEPS_FULL, bloch=bloch, seconds=secs)
    print(f"wrote {path} ({secs:.0f} s of reference run)")


if __name__ == "__main__":
    main()
