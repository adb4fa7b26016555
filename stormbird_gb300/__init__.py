"""stormbird_gb300 — GB300 (sm_103a) implementation of Stormbird's lifting-line hot path.

`Simulation` mirrors the reference's pystormbird class; all computation runs in the
CUDA library behind include/stormbird_gb300.h (built by `stormbird_gb300.build`).
"""
from ._abi import SbError, SimulationResult  # noqa: F401
from .batch import Batch  # noqa: F401
from .complete_sail_model import CompleteSailModel  # noqa: F401
from .simulation import Simulation  # noqa: F401

__all__ = ["Simulation", "Batch", "CompleteSailModel", "SimulationResult", "SbError"]
