"""GB300-native FDTD stepping engine with Meep's stepping API.

The compute path is the CUDA engine in meep_gb300/lib/libmfd.so (C ABI:
include/mfd.h); the C++ drop-in for meep::structure / meep::fields is
include/meep_gb300/meep.hpp over meep_gb300/lib/libmeep_gb300.so.  This package
binds the C ABI for Python (`Engine`, `Sim`) and carries the reference's
Python `Simulation` interface for the stepping path (meep_gb300.simulation,
re-exported here: `import meep_gb300 as mp; mp.Simulation(...)`).  There is no CPU fallback:
loading raises if the CUDA library has not been built.
"""
from ._lib import PRODUCT_LIB, Engine, MeepError, Sim, comp  # noqa: F401
from .simulation import (  # noqa: F401
    ALL, AUTOMATIC, Block, Bx, By, Bz, ContinuousSource, Cylinder, DrudeSusceptibility, Dx, Dy, Dz, Ex, Ey, Ez,
    EnergyRegion, Ldos, FluxData, FluxRegion, ForceData, NearToFarData, ForceRegion, GaussianSource, High, Hx, Hy, Hz, LorentzianSusceptibility, Low, MaterialGrid, Medium, Near2FarRegion, PML,
    Simulation, Source, Sphere, Vector3, Volume, X, Y, Z, after_time, air, at_beginning, at_end, at_every,
    dft_ldos, get_electric_energy, get_ldos_freqs, get_energy_freqs, get_flux_freqs, get_fluxes, get_magnetic_energy, get_total_energy, get_force_freqs, get_forces, get_near2far_freqs, inf, scale_flux_fields, scale_near2far_fields,
    stop_when_fields_decayed, vacuum)

__all__ = ["Engine", "Sim", "MeepError", "comp", "PRODUCT_LIB", "engine"]


def engine():
    """The CUDA engine (product library)."""
    return Engine(PRODUCT_LIB)
