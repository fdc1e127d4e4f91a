"""Flux data save / load (the reference's Python get_flux_data,
load_flux_data, load_minus_flux_data, scale_flux_fields; C ABI mfd_set_dft).

The usual reflection normalisation: run A without the scatterer and keep the
reflection plane's DFT sums; run B with the scatterer after
load_minus_flux_data, so that its plane accumulates the scattered fields
only; run C with the scatterer and nothing loaded.  B's sums must equal C's
minus A's, and B's flux must be the flux of those differences."""
import os

import numpy as np
import pytest

import meep_gb300 as mp


def relerr(a, b):
    """max |a - b| / max |b| over complex values"""
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape
    return float(np.abs(a - b).max() / np.abs(b).max())


def _run(lib, scatterer, load=None, minus=True):
    geometry = [mp.Block(mp.Vector3(0.6, 1.2, mp.inf), center=mp.Vector3(1.0, 0.1),
                         material=mp.Medium(epsilon=12))] if scatterer else []
    sim = mp.Simulation(cell_size=mp.Vector3(8, 4), resolution=10, geometry=geometry,
                        boundary_layers=[mp.PML(1.0)], eps_averaging=False,
                        sources=[mp.Source(mp.GaussianSource(0.5, fwidth=0.3), component=mp.Ez,
                                           center=mp.Vector3(-2.5), size=mp.Vector3(y=2))], _library=lib)
    refl = sim.add_flux(0.5, 0.3, 5, mp.FluxRegion(center=mp.Vector3(-1.5), size=mp.Vector3(y=2)))
    tran = sim.add_flux(0.5, 0.3, 5, mp.FluxRegion(center=mp.Vector3(2.5), size=mp.Vector3(y=2)))
    if load is not None:
        (sim.load_minus_flux_data if minus else sim.load_flux_data)(refl, load)
    sim.run(until_after_sources=20)
    return sim.get_flux_data(refl), np.array(mp.get_fluxes(refl)), np.array(mp.get_fluxes(tran))


def _check(lib, tol):
    a, fa, _ = _run(lib, False)
    c, fc, tc = _run(lib, True)
    b, fb, tb = _run(lib, True, load=a)
    assert relerr(b.E, c.E - a.E) <= tol and relerr(b.H, c.H - a.H) <= tol
    flux_of_diff = np.real(((c.E - a.E) * np.conj(c.H - a.H)).reshape(-1, 5)).sum(axis=0)
    assert relerr(fb, flux_of_diff) <= tol
    assert relerr(tb, tc) <= tol  # the transmission plane is untouched
    # the incident flux is positive at the reflection plane; the scattered
    # flux there runs back towards the source
    assert np.all(fa > 0) and np.all(fb < 0)
    # load_flux_data (no negation) then scale by -1 is load_minus_flux_data
    d, fd, _ = _run(lib, True, load=a, minus=False)
    assert relerr(d.E, c.E + a.E) <= tol


def test_flux_data_on_oracle(oracle_lib):
    _check(os.path.join(os.path.dirname(oracle_lib), "liboracle_meep.so"), 1e-12)


def test_load_rejects_wrong_size(oracle_lib):
    lib = os.path.join(os.path.dirname(oracle_lib), "liboracle_meep.so")
    a, _, _ = _run(lib, False)
    with pytest.raises(RuntimeError, match="does not agree"):
        _run(lib, True, load=mp.FluxData(E=a.E[:-1], H=a.H))


@pytest.mark.gpu
def test_flux_data_on_gpu(engine_lib):
    """The same workflow on the CUDA engine (FP64 and FP32 fields)."""
    from meep_gb300.simulation import PRODUCT_LIB
    _check(PRODUCT_LIB, 1e-12)
    _check(os.path.join(os.path.dirname(PRODUCT_LIB), "libmeep_gb300_single.so"), 1e-6)


def _run_fn(lib, scatterer, fload=None, nload=None):
    geometry = [mp.Block(mp.Vector3(0.6, 1.2, mp.inf), center=mp.Vector3(0.3, 0.1),
                         material=mp.Medium(epsilon=12))] if scatterer else []
    sim = mp.Simulation(cell_size=mp.Vector3(8, 6), resolution=10, geometry=geometry,
                        boundary_layers=[mp.PML(1.0)], eps_averaging=False,
                        sources=[mp.Source(mp.GaussianSource(0.5, fwidth=0.3), component=mp.Ez,
                                           center=mp.Vector3(-2.5), size=mp.Vector3(y=2))], _library=lib)
    force = sim.add_force(0.5, 0.3, 3, mp.ForceRegion(center=mp.Vector3(1.5), size=mp.Vector3(y=2), direction=mp.X),
                          mp.ForceRegion(center=mp.Vector3(0.3, 1.5), size=mp.Vector3(2), direction=mp.X))
    n2f = sim.add_near2far(0.5, 0.3, 3, mp.Near2FarRegion(center=mp.Vector3(2.5), size=mp.Vector3(y=3)))
    if fload is not None:
        sim.load_minus_force_data(force, fload)
    if nload is not None:
        sim.load_minus_near2far_data(n2f, nload)
    sim.run(until_after_sources=10)
    ff = sim.get_farfields_at(n2f, [[30.0, 5.0, 0.0], [40.0, -10.0, 0.0]])
    return sim.get_force_data(force), sim.get_near2far_data(n2f), ff


def test_force_and_near2far_data_on_oracle(oracle_lib):
    """get/load_minus force and near2far data: the loaded-negated run holds
    the difference of the separate runs' sums, and (the near-to-far transform
    being linear in them) its far fields are the difference of theirs."""
    lib = os.path.join(os.path.dirname(oracle_lib), "liboracle_meep.so")
    fa, na, ffa = _run_fn(lib, False)
    fc, nc, ffc = _run_fn(lib, True)
    fb, nb, ffb = _run_fn(lib, True, fload=fa, nload=na)
    for k in ("offdiag1", "offdiag2", "diag"):
        assert getattr(fa, k).size > 0
        assert relerr(getattr(fb, k), getattr(fc, k) - getattr(fa, k)) <= 1e-12, k
    assert relerr(nb.F, nc.F - na.F) <= 1e-12
    assert relerr(ffb, ffc - ffa) <= 1e-12


def test_abi_errors(oracle_lib):
    """The C ABI refuses a 1-D far field, an unknown monitor for mfd_set_dft,
    an unknown source for mfd_src_current, and an include_weights mode other
    than 0, 1, 2, each with a message."""
    import ctypes as C
    from meep_gb300 import _lib
    eng = _lib.Engine(oracle_lib)
    s = _lib.Sim(eng, 1, (0, 0, 20), (0, 0, -20), 10.0, components=[0, 4, 6, 10])
    w = [None, None, np.ones(3)]
    mid = s.add_dft(0, [0, 0, 5], [0, 0, 7], w, centered=False, freqs=[0.5])
    with pytest.raises(_lib.MeepError, match="only 2d or 3d"):
        s.farfield([(mid, 4, [0, 0, 0], [0, 0, 0])], [[0, 0, 1.0]])
    buf = np.zeros(6)
    assert eng.lib.mfd_set_dft(s.h, 99, buf.ctypes.data_as(C.POINTER(C.c_double))) != 0
    assert b"unknown monitor" in eng.lib.mfd_last_error()
    out = np.zeros(2)
    assert eng.lib.mfd_src_current(s.h, 0, 1.0, out.ctypes.data_as(C.POINTER(C.c_double))) != 0
    assert b"unknown source" in eng.lib.mfd_last_error()
    with pytest.raises(_lib.MeepError, match="include_weights"):
        s.add_dft(0, [0, 0, 5], [0, 0, 7], w, include_weights=3, centered=False, freqs=[0.5])
