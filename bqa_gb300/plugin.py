"""Registration of the GB300 backend into an installed ``bqa`` package.

The reference selects a backend by the config's ``"backend"`` string, looked up in
``bqa.backends.BACKEND_STR_TO_BACKEND`` (``src/bqa/backends.py:26``; validated in
``src/bqa/config/config_syntax.py:63-70``, used in
``src/bqa/config/config_canonicalization.py:211``).  Its numpy and CuPy backends implement
the per-operation ``Tensor`` ABC and are driven one batched op at a time by the state VM
(``src/bqa/state.py``).  The GB300 backend fuses whole phases of an annealing step into
kernels (one launch per degree class per phase), so it sits one level higher: it is the
``run_qa`` implementation for configs whose backend is ``"gb300"``.

``register()`` makes that selection work inside bqa itself:

* ``"gb300"`` is added to the registry, so bqa's config validation accepts it;
* ``bqa.run_qa`` / ``bqa.core.run_qa`` are wrapped so a config with ``"backend": "gb300"``
  runs through ``bqa_gb300.run_qa`` (same config dict in, same result list out); every other
  config goes to the original function unchanged.

The registry entry is a marker class: bqa's per-operation code paths (``config_to_context``
followed by the state VM) cannot drive a fused backend, and calling its tensor constructors
raises with a pointer to ``run_qa``.
"""
from __future__ import annotations

import functools
import importlib

BACKEND_NAME = "gb300"


class GB300BackendMarker:
    """Registry entry for ``"gb300"`` in bqa's backend table."""

    @classmethod
    def _fused_only(cls, *_, **__):
        raise NotImplementedError(
            "the gb300 backend runs whole annealing steps as fused kernels; "
            "use bqa.run_qa / bqa_gb300.run_qa with config['backend'] = 'gb300'")

    make_from_list = make_from_numpy = make_from_raw_tensor = make_constant = make_empty = _fused_only


def _wrap(original):
    if getattr(original, "_bqa_gb300_wrapped", False):
        return original

    @functools.wraps(original)
    def run_qa(config, *args, **kwargs):
        if isinstance(config, dict) and config.get("backend") == BACKEND_NAME:
            from .core import run_qa as gb300_run_qa
            return gb300_run_qa(config)
        return original(config, *args, **kwargs)

    run_qa._bqa_gb300_wrapped = True
    return run_qa


def register() -> bool:
    """Install the backend into an importable ``bqa``; returns False if bqa is absent."""
    try:
        bqa = importlib.import_module("bqa")
        backends = importlib.import_module("bqa.backends")
        core = importlib.import_module("bqa.core")
    except ImportError:
        return False
    backends.BACKEND_STR_TO_BACKEND[BACKEND_NAME] = GB300BackendMarker
    core.run_qa = _wrap(core.run_qa)
    bqa.run_qa = _wrap(bqa.run_qa)
    return True
