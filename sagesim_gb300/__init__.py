"""GB300-native engine for SAGESim's per-tick agent step.

The public API mirrors SAGESim's (`Breed`, `Model`, `NetworkSpace`) for the
per-tick step on a network; the work runs in hand-written sm_103a CUDA kernels
behind the C ABI of include/sagesim_gb300.h.
"""
from ._native import SageSimError  # noqa: F401
from .breed import Breed  # noqa: F401
from .engine import Engine  # noqa: F401
from .model import Model  # noqa: F401
from .space import NetworkSpace  # noqa: F401
from .steps import CudaStep, OpinionStep, SIRStep  # noqa: F401

__version__ = "0.1.0"
__all__ = ["Model", "Breed", "NetworkSpace", "SIRStep", "OpinionStep", "CudaStep", "Engine",
           "SageSimError"]
