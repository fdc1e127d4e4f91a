"""Divergence test of fields::step(): the reference aborts with "simulation
fields are NaN or Inf" when the electric energy density at the cell centre
stops being finite (src/step.cpp:137-138).  A NaN permittivity at the centre
makes E = chi1inv D non-finite on the first step (0 * NaN), as a diverging
run eventually does.

CPU: the oracle checks every step, as the reference does; the Python front
end raises the reference's RuntimeError text.
GPU: the CUDA engine probes the centre every MFD_FINITE_CHECK_EVERY steps
(default 16) into host-mapped memory and raises at the next step or
synchronisation, so a run stops at most that many steps after the
reference would."""
import math
import os

import numpy as np
import pytest

from meep_gb300 import _lib
import meep_gb300 as mp

MSG = "meep: simulation fields are NaN or Inf"


def _problem(lib, nan_at_centre=True, precision=64):
    """3-D 24 x 20 x 22 cells with PML, random eps, an Ex point source off
    the centre; optionally eps = NaN at the centre point of every E
    component."""
    eng = _lib.Engine(lib)
    rng = np.random.default_rng(5)
    n = (24, 20, 22)
    comps = [_lib.comp(t, d) for t in range(4) for d in range(3)]
    pml = {(d, s): (0.5, 1e-15, 1.0) for d in range(3) for s in range(2)}
    sim = _lib.Sim(eng, dim=3, n=n, io=[-x for x in n], a=10.0, pml=pml, precision=precision, components=comps)
    shape = tuple(sim.ext)
    for d in range(3):
        chi = 1.0 / rng.uniform(1.0, 4.0, size=shape)
        if nan_at_centre:
            chi[n[0] // 2 - 1:n[0] // 2 + 1, n[1] // 2 - 1:n[1] // 2 + 1, n[2] // 2 - 1:n[2] // 2 + 1] = np.nan
        sim.set_chi1inv(_lib.comp(_lib.E, d), d, chi)
    src = sim.add_gaussian_src(0.5, 0.5)
    sim.add_source_points(_lib.comp(_lib.E, 0), src, [int(np.ravel_multi_index((5, 6, 7), shape))], [1.0])
    return sim


def _steps_until_error(sim, limit):
    for k in range(1, limit + 1):
        try:
            sim.step(1)
        except _lib.MeepError as e:
            assert str(e) == MSG, str(e)
            return k
    return None


def test_oracle_stops_on_first_step(oracle_lib):
    sim = _problem(oracle_lib)
    assert _steps_until_error(sim, 5) == 1


def test_oracle_finite_run_continues(oracle_lib):
    sim = _problem(oracle_lib, nan_at_centre=False)
    sim.step(40)
    assert np.isfinite(sim.get_field(_lib.comp(_lib.E, 0))).all()


def test_simulation_front_end_raises(oracle_lib):
    """meep_gb300.Simulation.run raises the reference's RuntimeError (the
    SWIG layer maps meep::abort to RuntimeError, python/meep.i:1365-1380)."""
    lib = os.path.join(os.path.dirname(oracle_lib), "liboracle_meep.so")
    sim = mp.Simulation(cell_size=mp.Vector3(6, 4), resolution=10, boundary_layers=[mp.PML(1.0)],
                        geometry=[mp.Block(mp.Vector3(0.5, 0.5, mp.inf), material=mp.Medium(epsilon=math.nan))],
                        eps_averaging=False,
                        sources=[mp.Source(mp.GaussianSource(0.3, fwidth=0.2), component=mp.Ez,
                                           center=mp.Vector3(-2))], _library=lib)
    with pytest.raises(RuntimeError, match="simulation fields are NaN or Inf"):
        sim.run(until=5)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [64, 32])
def test_gpu_stops_within_check_interval(precision, engine_lib):
    sim = _problem(engine_lib, precision=precision)
    k = _steps_until_error(sim, 40)
    assert k is not None and k <= 16, k


@pytest.mark.gpu
def test_gpu_check_every_step(engine_lib, monkeypatch):
    monkeypatch.setenv("MFD_FINITE_CHECK_EVERY", "1")
    sim = _problem(engine_lib)
    assert _steps_until_error(sim, 5) == 1


@pytest.mark.gpu
def test_gpu_batched_steps_raise(engine_lib):
    """one mfd_step call of many steps: the flag is read after the batch"""
    sim = _problem(engine_lib)
    with pytest.raises(_lib.MeepError, match="NaN or Inf"):
        sim.step(50)


@pytest.mark.gpu
def test_gpu_finite_run_continues(engine_lib):
    sim = _problem(engine_lib, nan_at_centre=False)
    sim.step(64)
    assert np.isfinite(sim.get_field(_lib.comp(_lib.E, 0))).all()
