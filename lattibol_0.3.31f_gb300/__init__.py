"""GB300-native lattice Boltzmann hot path of lattibol.

The compute lives in liblbgb300.so (hand-written CUDA for sm_103a behind a C
ABI, see include/lbgb300.h).  This package only loads it and mirrors the
reference's host-side interface for Python callers; it has no CPU fallback.
"""
from . import abi  # noqa: F401

_lib = None


def lib():
    """The loaded liblbgb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        _lib = abi.load()
    return _lib


from .lattice import (DeviceData, Ensemble, Lattice, LBError, W2, W3,  # noqa: E402,F401
                      droplet_ensemble)
from . import closure  # noqa: E402,F401
from . import slab  # noqa: E402,F401
from . import case  # noqa: E402,F401
from .case import Input, Output, SimulationD2Q9, SimulationD3Q19  # noqa: E402,F401
