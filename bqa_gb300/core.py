"""``run_qa`` of the GB300 backend: same job dict in, same result list out as the reference.

Mirrors ``src/bqa/core.py:13-35``: the config is analysed and compiled into degree classes,
the state is initialised on the GPU, and the instruction list is executed in order --
evolution dicts run one annealing step each, ``"get_bloch_vectors"`` appends
``["bloch_vectors", [[x, y, z], ...]]`` and ``"measure"`` appends
``["measurement_outcomes", [+1/-1, ...]]``.
"""
from __future__ import annotations

import logging

import numpy as np

from . import config as cfg
from .engine import Annealer
from .layout import build_context

log = logging.getLogger(__name__)


def run_qa(config, device=None, as_arrays: bool = False) -> list:
    """Run a job; with ``as_arrays`` the result values stay numpy arrays (n x 3 float64 Bloch
    vectors, n int64 outcomes) instead of nested lists."""
    import torch
    on_gpu = torch.cuda.is_available()
    ctx = build_context(config, layout_device=(device if device is not None else "cuda") if on_gpu else None)
    log.info("Context is built")
    return run_compiled(ctx, device=device, as_arrays=as_arrays)


def run_compiled(ctx, device=None, as_arrays: bool = False) -> list:
    """Execute the instruction list of a compiled context (``layout.Context``) on the GPU."""
    job = Annealer(ctx, device=device)
    total = len(ctx.instructions)
    out = []
    for num, ins in enumerate(ctx.instructions):
        log.info(f"Instruction number {num} / {total} started")
        if isinstance(ins, dict):
            job.run_layer(ins["xtime"], ins["ztime"])
        elif ins == cfg.MEASURE:
            outcomes = job.measure()
            out.append(["measurement_outcomes", np.asarray(outcomes, dtype=np.int64) if as_arrays else outcomes])
        elif ins == cfg.GET_BLOCH_VECTORS:
            bloch = job.bloch_vectors()
            out.append(["bloch_vectors", bloch if as_arrays else bloch.tolist()])
        else:
            raise ValueError(f"Unknown instruction {ins}")
    # a tensor-core CTA whose bounded wait for its MMAs ran out voids the results (never in
    # correct operation; the counter is read and reset once per job)
    faults = job.lib.tc_faults(job.stream)
    if faults:
        raise RuntimeError(f"{faults} tensor-core CTA(s) timed out waiting for their MMAs; results are void")
    return out
