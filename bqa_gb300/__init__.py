"""GB300-native (sm_103a) backend for bqa's belief-propagation tensor-network annealer.

``run_qa(config)`` takes the reference's job dict and returns its result list; the
``Annealer`` class exposes the step-level API (run_layer, run_bp, densities, <ZZ>, energy,
measurement) of one job resident on one GPU.
"""
from .config import ConfigSyntaxError  # noqa: F401
from .core import run_qa  # noqa: F401
from .engine import Annealer  # noqa: F401

__version__ = "0.1.0"
