"""Generate golden fixtures by running the REFERENCE bqa (v0.1.6) numpy backend at FP64.

Run where the reference sources are available, with BQA_REFERENCE_SRC naming the
reference's ``src`` directory:

    BQA_REFERENCE_SRC=<reference checkout>/src python tests/golden/make_golden.py [--big]

It imports the reference through a stub dist-info (its ``__init__`` asks importlib.metadata
for its version), runs ``bqa.run_qa`` / the state-VM phase functions on seeded small
problems and writes ``tests/golden/*.npz`` + ``cases.json``.  The GPU tests and the oracle
tests read only those files; nothing at test time imports the reference.

``--big`` also records the full CPU headline case (n=1000 random 3-regular, chi=4, 100
steps; about 25 s of CPU).
"""
from __future__ import annotations

import json
import os
import random
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def _reference_src() -> Path:
    src = os.environ.get("BQA_REFERENCE_SRC")
    if not src or not (Path(src) / "bqa").is_dir():
        raise SystemExit("set BQA_REFERENCE_SRC to the reference bqa checkout's src directory")
    return Path(src)


def _import_reference():
    ref_src = _reference_src()
    shim = Path(tempfile.mkdtemp(prefix="bqa_shim_"))
    info = shim / "bqa-0.1.6.dist-info"
    info.mkdir()
    (info / "METADATA").write_text("Metadata-Version: 2.1\nName: bqa\nVersion: 0.1.6\n")
    os.environ["BQA_PRECISION"] = "double"
    sys.path[:0] = [str(shim), str(ref_src)]
    import bqa  # noqa: F401
    import bqa.state as st
    from bqa.config.core import config_to_context
    from bqa.core import run_qa
    return st, config_to_context, run_qa


def random_regular_edges(n: int, d: int, seed: int) -> list:
    """Edge list of a seeded random d-regular graph (networkx, as the reference uses)."""
    import networkx as nx
    g = nx.random_regular_graph(d, n, random.Random(seed))
    g = nx.convert_node_labels_to_integers(g)
    return [list(e) for e in g.edges]


def mixed_degree_edges(n: int, p: float, seed: int) -> list:
    import networkx as nx
    g = nx.gnp_random_graph(n, p, seed=seed)
    # keep it connected enough: add a ring so that no node is isolated
    for v in range(n):
        g.add_edge(v, (v + 1) % n)
    return [list(e) for e in g.edges]


def grid_edges(m: int, k: int) -> list:
    import networkx as nx
    g = nx.convert_node_labels_to_integers(nx.grid_2d_graph(m, k))
    return [list(e) for e in g.edges]


def make_config(edges, fields, chi, steps, total_time, **kw) -> dict:
    cfg = {
        "nodes": {int(v): float(h) for v, h in fields.items()},
        "edges": {(int(a), int(b)): float(J) for a, b, J in edges},
        "max_bond_dim": chi,
        "bp_eps": kw.get("bp_eps", 1e-9),
        "pinv_eps": kw.get("pinv_eps", 1e-6),
        "max_bp_iter_number": kw.get("max_bp_iter_number", 200),
        "damping": kw.get("damping", 0.0),
        "seed": kw.get("seed", 42),
        "backend": "numpy",
        "schedule": {
            "total_time": total_time,
            "starting_mixing": 1.0,
            "actions": kw.get("actions", [{"weight": 1.0, "steps_number": steps, "final_mixing": 0.0},
                                          "get_bloch_vectors"]),
        },
    }
    return cfg


def to_json_config(cfg: dict) -> dict:
    out = dict(cfg)
    out["nodes"] = [[v, h] for v, h in cfg["nodes"].items()]
    out["edges"] = [[a, b, J] for (a, b), J in cfg["edges"].items()]
    return out


def cases(big: bool):
    rng = np.random.default_rng(7)
    out = {}
    # 9-node tree of the reference's own BP tests (tests/test_core_subroutines.py:176-189)
    tree = {"nodes": {1: 0.3, 3: -0.7, 5: 1.0, 6: -1.0, 7: 0.25},
            "edges": {(2, 0): 1.0, (1, 2): -1.0, (2, 4): 0.5, (4, 3): -0.5, (4, 5): 0.75,
                      (4, 6): -0.75, (6, 7): 0.3, (8, 6): 0.6},
            "default_field": 0.6, "bp_eps": 1e-10, "pinv_eps": 1e-7, "max_bond_dim": 4,
            "backend": "numpy",
            "schedule": {"total_time": 3.0, "starting_mixing": 1.0,
                         "actions": [{"weight": 1.0, "steps_number": 12, "final_mixing": 0.0},
                                     "get_bloch_vectors"]}}
    out["tree9"] = tree
    e = random_regular_edges(16, 3, 1)
    out["rr3_n16_chi4"] = make_config([(a, b, rng.normal()) for a, b in e],
                                      {v: rng.normal() for v in range(16)}, 4, 30, 3.0)
    e = random_regular_edges(24, 3, 2)
    out["rr3_n24_chi8"] = make_config([(a, b, 2 * int(rng.integers(0, 2)) - 1) for a, b in e],
                                      {v: rng.uniform(-0.5, 0.5) for v in range(24)}, 8, 24, 2.4,
                                      bp_eps=1e-8, max_bp_iter_number=80)
    e = mixed_degree_edges(18, 0.15, 3)
    out["mixed_n18_chi3"] = make_config([(a, b, rng.normal()) for a, b in e],
                                        {v: rng.normal(0, 0.3) for v in range(18)}, 3, 16, 2.0)
    e = grid_edges(3, 4)
    out["grid3x4_chi4_damped"] = make_config([(a, b, rng.normal()) for a, b in e],
                                             {v: rng.normal() for v in range(12)}, 4, 15, 2.0,
                                             damping=0.3, max_bp_iter_number=6, bp_eps=1e-7)
    e = random_regular_edges(12, 3, 4)
    out["rr3_n12_measure"] = make_config(
        [(a, b, rng.normal()) for a, b in e], {v: rng.normal() for v in range(12)}, 4, 20, 4.0,
        bp_eps=1e-8, seed=5,
        actions=[{"weight": 1.0, "steps_number": 20, "final_mixing": 0.0}, "get_bloch_vectors", "measure"])
    e = random_regular_edges(20, 4, 5)
    out["rr4_n20_chi4"] = make_config([(a, b, rng.normal()) for a, b in e],
                                      {v: 0.0 for v in range(20)}, 4, 12, 1.5, bp_eps=1e-8)
    if big:
        r = random.Random(0)
        import networkx as nx
        g = nx.convert_node_labels_to_integers(nx.random_regular_graph(3, 1000, r))
        nodes = {v: r.gauss(0, 1) for v in g.nodes}
        edges = {ed: r.gauss(0, 1) for ed in g.edges}
        out["c1_rr3_n1000_chi4"] = {
            "nodes": nodes, "edges": edges, "max_bond_dim": 4, "bp_eps": 1e-6, "pinv_eps": 1e-6,
            "max_bp_iter_number": 100, "backend": "numpy",
            "schedule": {"total_time": 10.0, "starting_mixing": 1.0,
                         "actions": [{"weight": 1.0, "steps_number": 100, "final_mixing": 0.0},
                                     "get_bloch_vectors"]}}
    return out


def main() -> None:
    big = "--big" in sys.argv
    st, config_to_context, run_qa = _import_reference()
    import logging
    logging.basicConfig(level=logging.ERROR)
    manifest = {}
    for name, cfg in cases(big).items():
        t0 = time.perf_counter()
        ctx = config_to_context(cfg)
        state = st._initialize_state(ctx)
        dims = []
        results = []
        for ins in ctx.instructions:
            if isinstance(ins, dict):
                st.run_layer(ctx, ins["xtime"], ins["ztime"], state)
                dims.append(state.bond_dim)
            elif ins == "get_bloch_vectors":
                from bqa.utils import convert_density_matrix_to_bloch_vector
                dens = st.get_density_matrices(ctx, state)
                results.append(("bloch_vectors", np.array([convert_density_matrix_to_bloch_vector(x) for x in dens])))
            elif ins == "measure":
                results.append(("measurement_outcomes", np.array(st.measure(ctx, state))))
        arrays = {"dims": np.array(dims), "lmbds": state.lmbds.numpy.real}
        for i, (kind, val) in enumerate(results):
            arrays[f"result{i}_{kind}"] = val
        np.savez_compressed(HERE / f"{name}.npz", **arrays)
        manifest[name] = {"config": to_json_config(cfg), "results": [k for k, _ in results],
                          "seconds": round(time.perf_counter() - t0, 2)}
        print(name, "done in", manifest[name]["seconds"], "s, final dim", dims[-1] if dims else None)
    with open(HERE / "cases.json", "w") as f:
        json.dump(manifest, f, indent=1)


if __name__ == "__main__":
    main()
