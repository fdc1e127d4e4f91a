"""CPU: the C-ABI libraries load and export every entry point of include/mfd.h;
host-side validation errors surface as exceptions (no GPU needed)."""
import ctypes
import os
import re

import pytest

from meep_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "mfd.h")).read()
    return sorted(set(re.findall(r"\b(mfd_[a-z_0-9]+)\s*\(", text)))


def test_header_and_binding_agree():
    names = {n for n, _, _ in _lib.SIGNATURES}
    assert set(declared_symbols()) == names


def test_product_library_exports(engine_lib):
    lib = ctypes.CDLL(engine_lib)
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_oracle_library_exports(oracle_lib):
    lib = ctypes.CDLL(oracle_lib)
    for name in declared_symbols():
        if name not in _lib.DEVICE_ONLY:
            assert hasattr(lib, name), name


def test_errors_are_reported(oracle_lib):
    eng = _lib.Engine(oracle_lib)
    with pytest.raises(_lib.MeepError, match="dim must be"):
        _lib.Sim(eng, dim=4, n=(4, 4, 4), io=(0, 0, 0), a=10)
    with pytest.raises(_lib.MeepError, match="PML slabs"):
        _lib.Sim(eng, dim=2, n=(10, 10, 0), io=(0, 0, 0), a=10, pml={(0, 0): (1.0, 1e-15, 1.0)},
                 components=[0])
    sim = _lib.Sim(eng, dim=2, n=(10, 10, 0), io=(0, 0, 0), a=10,
                   components=[_lib.comp(_lib.E, 2), _lib.comp(_lib.D, 2)])
    with pytest.raises(_lib.MeepError, match="out of range"):
        sim.add_source_points(_lib.comp(_lib.E, 2), sim.add_gaussian_src(0.1, 0.1), [10**6], [1.0])
