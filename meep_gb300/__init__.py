"""GB300-native FDTD stepping engine with Meep's stepping API.

The compute path is the CUDA engine in meep_gb300/lib/libmfd.so (C ABI:
include/mfd.h); the C++ drop-in for meep::structure / meep::fields is
include/meep_gb300/meep.hpp over meep_gb300/lib/libmeep_gb300.so.  This package
binds the C ABI for Python (`Engine`, `Sim`).  There is no CPU fallback:
loading raises if the CUDA library has not been built.
"""
from ._lib import PRODUCT_LIB, Engine, MeepError, Sim, comp  # noqa: F401

__all__ = ["Engine", "Sim", "MeepError", "comp", "PRODUCT_LIB", "engine"]


def engine():
    """The CUDA engine (product library)."""
    return Engine(PRODUCT_LIB)
