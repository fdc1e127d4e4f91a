"""Energy density spectra (dft_energy, src/dft.cpp:681-750).

Case py_energy of tests/golden/golden_driver.cpp restates the reference's
python/tests/test_dft_energy.py (an eps = 12 slab guide, flux and energy
monitors across it at decimation 1 and 10) with a line source in place of the
eigenmode source; records the flux and the electric, magnetic and total
energies."""
import os

import pytest

from harness import GPU_DRIVER, ORACLE_DRIVER, golden, run_driver

KEYS = ["flux", "electric", "magnetic", "total", "electric_dec", "magnetic_dec", "total_dec"]


def _check(out, ref, tol):
    assert out["t"][0] == ref["t"][0]
    for k in KEYS:
        assert abs(out[k][0] - ref[k][0]) <= tol * abs(ref[k][0]), (k, out[k][0], ref[k][0])


def test_fixture_relations():
    """As the reference test asserts: electric + magnetic = total (7 places)
    and decimation 10 agrees with decimation 1 (1 place)."""
    ref = golden("py_energy", "f64")
    assert round(ref["electric"][0] + ref["magnetic"][0] - ref["total"][0], 7) == 0
    for k in ("electric", "magnetic"):
        assert round(ref[k][0] - ref[k + "_dec"][0], 1) == 0


def test_oracle_fp64_matches_reference(oracle_lib, tmp_path):
    _check(run_driver(ORACLE_DRIVER[64], "py_energy", tmp_path), golden("py_energy", "f64"), 1e-13)


def script_energy(lib):
    import meep_gb300 as mp
    sim = mp.Simulation(resolution=10, cell_size=mp.Vector3(10, 5), eps_averaging=False,
                        geometry=[mp.Block(size=mp.Vector3(mp.inf, 1, mp.inf), material=mp.Medium(epsilon=12))],
                        boundary_layers=[mp.PML(1)],
                        sources=[mp.Source(mp.GaussianSource(0.15, fwidth=0.03), component=mp.Ez,
                                           center=mp.Vector3(-3), size=mp.Vector3(y=5))], _library=lib)
    flux = sim.add_flux(0.15, 0, 1, mp.FluxRegion(center=mp.Vector3(3), size=mp.Vector3(y=5)), decimation_factor=1)
    energy = sim.add_energy(0.15, 0, 1, mp.EnergyRegion(center=mp.Vector3(3), size=mp.Vector3(y=5)),
                            decimation_factor=1)
    energy_dec = sim.add_energy(0.15, 0, 1, mp.EnergyRegion(center=mp.Vector3(3), size=mp.Vector3(y=5)),
                                decimation_factor=10)
    sim.run(until_after_sources=50)
    assert mp.get_energy_freqs(energy) == [0.15]
    out = {"flux": mp.get_fluxes(flux), "t": [sim.meep_time()]}
    for suffix, e in (("", energy), ("_dec", energy_dec)):
        out["electric" + suffix] = mp.get_electric_energy(e)
        out["magnetic" + suffix] = mp.get_magnetic_energy(e)
        out["total" + suffix] = mp.get_total_energy(e)
    return out


def test_python_script_on_oracle(oracle_lib):
    """add_energy and get_*_energy in the Python front end reproduce the
    reference core's run of the script within 1e-12."""
    _check(script_energy(os.path.join(os.path.dirname(oracle_lib), "liboracle_meep.so")),
           golden("py_energy", "f64"), 1e-12)


@pytest.mark.gpu
def test_gpu_matches_reference(gpu_drivers, tmp_path):
    """CUDA engine: FP64 within 1e-10 of the reference, FP32 within 1e-5;
    the Python script on the GPU within 1e-10."""
    ref = golden("py_energy", "f64")
    _check(run_driver(GPU_DRIVER[64], "py_energy", tmp_path), ref, 1e-10)
    _check(run_driver(GPU_DRIVER[32], "py_energy", tmp_path), ref, 1e-5)
    from meep_gb300.simulation import PRODUCT_LIB
    _check(script_energy(PRODUCT_LIB), ref, 1e-10)
