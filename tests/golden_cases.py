"""Loader for the golden fixtures recorded from the reference (see golden/make_golden.py)."""
import json
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"


def manifest() -> dict:
    with open(GOLDEN / "cases.json") as f:
        return json.load(f)


def case_names(max_nodes: int | None = None) -> list:
    out = []
    for name, entry in manifest().items():
        cfg = entry["config"]
        n = 1 + max(max(max(a, b) for a, b, _ in cfg["edges"]), max((v for v, _ in cfg["nodes"]), default=-1))
        if max_nodes is None or n <= max_nodes:
            out.append(name)
    return out


def config(name: str, backend: str | None = None) -> dict:
    cfg = dict(manifest()[name]["config"])
    cfg["nodes"] = {int(v): float(h) for v, h in cfg["nodes"]}
    cfg["edges"] = {(int(a), int(b)): float(J) for a, b, J in cfg["edges"]}
    if backend is None:
        cfg.pop("backend", None)
    else:
        cfg["backend"] = backend
    return cfg


def arrays(name: str) -> dict:
    with np.load(GOLDEN / f"{name}.npz") as z:
        return {k: z[k] for k in z.files}
