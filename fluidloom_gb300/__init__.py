"""fluidloom_gb300 — GB300-native AMR lattice-Boltzmann hot path.

Python view of the C ABI (include/fluidloom_gb300.h).  All compute runs in the
sm_103a CUDA library built in-tree; importing this package never falls back to
a CPU path.
"""
from . import _capi  # noqa: F401
from .runtime import Context, DeviceArray, FluidLoomError, check  # noqa: F401

__all__ = ["Context", "DeviceArray", "FluidLoomError", "check"]
