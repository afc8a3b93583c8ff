"""GB300-native (sm_103a) backend for bqa's belief-propagation tensor-network annealer."""
from .config import ConfigSyntaxError  # noqa: F401

__version__ = "0.1.0"
