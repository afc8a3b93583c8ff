"""``run_qa`` of the GB300 backend: same job dict in, same result list out as the reference.

Mirrors ``src/bqa/core.py:13-35``: the config is analysed and compiled into degree classes,
the state is initialised on the GPU, and the instruction list is executed in order --
evolution dicts run one annealing step each, ``"get_bloch_vectors"`` appends
``["bloch_vectors", [[x, y, z], ...]]`` and ``"measure"`` appends
``["measurement_outcomes", [+1/-1, ...]]``.
"""
from __future__ import annotations

import logging

from . import config as cfg
from .engine import Annealer
from .layout import build_context

log = logging.getLogger(__name__)


def run_qa(config, device=None) -> list:
    ctx = build_context(config)
    log.info("Context is built")
    job = Annealer(ctx, device=device)
    total = len(ctx.instructions)
    out = []
    for num, ins in enumerate(ctx.instructions):
        log.info(f"Instruction number {num} / {total} started")
        if isinstance(ins, dict):
            job.run_layer(ins["xtime"], ins["ztime"])
        elif ins == cfg.MEASURE:
            out.append(["measurement_outcomes", job.measure()])
        elif ins == cfg.GET_BLOCH_VECTORS:
            out.append(["bloch_vectors", job.bloch_vectors().tolist()])
        else:
            raise ValueError(f"Unknown instruction {ins}")
    return out
