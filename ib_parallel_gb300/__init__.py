"""GB300-native immersed-boundary time step (drop-in for IB_Parallel's Fortran
time-step modules).  The compute path is the CUDA library ``libibgpu.so`` built
from ``csrc/`` for sm_103a; this package only binds it."""
from .ibgpu import (Body, IbError, Params, Simulation, load, EXPORTS, LIB_PATH)  # noqa: F401
from . import geometry  # noqa: F401

__all__ = ["Body", "Params", "Simulation", "IbError", "load", "EXPORTS", "LIB_PATH", "geometry"]
