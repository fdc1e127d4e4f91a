"""Maxwell-stress force (dft_force, src/stress.cpp).

Case py_force of tests/golden/golden_driver.cpp restates the reference's
python/tests/test_force.py through the C++ calls its Python layer makes: a
2-D Ez pulse in vacuum, a force region along y across the cell (diagonal
stress terms: square-root dV weights and +-1/2 extra weights) at decimation 1
and 10, and the test's 2 x 2 box of x-force regions (off-diagonal terms on
two sides), run until the field at the source has decayed by 1e-6
(stop_when_fields_decayed).  Records: the three forces, the stop time and Ez.
"""
import numpy as np
import pytest

from harness import GPU_DRIVER, ORACLE_DRIVER, golden, run_driver

# the reference test's golden master (assertAlmostEqual, 7 places)
REFERENCE_FORCE = -0.11039089113393187


def _check(out, ref, rel, box_abs, fields_equal):
    assert out["t"][0] == ref["t"][0]
    for k in ("force", "force_dec"):
        assert abs(out[k][0] - ref[k][0]) <= rel * abs(ref[k][0]), (k, out[k][0], ref[k][0])
    # the box encloses the source symmetrically: its net force is zero up to
    # rounding, so it is compared in absolute terms against the line force
    assert abs(out["force_box"][0] - ref["force_box"][0]) <= box_abs * abs(ref["force"][0]), out["force_box"]
    if fields_equal:
        assert np.array_equal(np.asarray(out["Ez"]), np.asarray(ref["Ez"]))


def test_fixture_matches_reference_golden_master():
    """The restated script, run by the reference core, gives the reference
    test's own golden master to 7 places (observed 1e-16): the fixture pins
    the restatement."""
    ref = golden("py_force", "f64")
    assert round(ref["force"][0] - REFERENCE_FORCE, 7) == 0
    assert round(ref["force"][0] - ref["force_dec"][0], 7) == 0


def test_oracle_fp64_matches_reference(oracle_lib, tmp_path):
    """CPU restatement: fields bit-identical, same stop step, forces within
    1e-13 (the per-pair reduction adds in another order)."""
    _check(run_driver(ORACLE_DRIVER[64], "py_force", tmp_path), golden("py_force", "f64"), 1e-13, 1e-13, True)


def script_force(lib):
    """The reference's test_force through the Python front end."""
    import meep_gb300 as mp
    sim = mp.Simulation(resolution=20, cell_size=mp.Vector3(10, 10), boundary_layers=[mp.PML(1.0)],
                        sources=[mp.Source(src=mp.GaussianSource(frequency=1.0, fwidth=1.0), center=mp.Vector3(),
                                           component=mp.Ez)], _library=lib)
    fr = mp.ForceRegion(center=mp.Vector3(0, 1.27), direction=mp.Y, size=mp.Vector3(4.38, 0))
    fr_box = [mp.ForceRegion(direction=mp.X, center=mp.Vector3(1.0, 0, 0), size=mp.Vector3(0, 2.0, 0), weight=1.0),
              mp.ForceRegion(direction=mp.X, center=mp.Vector3(-1.0, 0, 0), size=mp.Vector3(0, 2.0, 0), weight=-1.0),
              mp.ForceRegion(direction=mp.X, center=mp.Vector3(0, 1.0, 0), size=mp.Vector3(2.0, 0, 0), weight=1.0),
              mp.ForceRegion(direction=mp.X, center=mp.Vector3(0, -1.0, 0), size=mp.Vector3(2.0, 0, 0), weight=-1.0)]
    force = sim.add_force(1.0, 0, 1, fr, decimation_factor=1)
    force_dec = sim.add_force(1.0, 0, 1, fr, decimation_factor=10)
    force_box = sim.add_force(1.0, 0, 1, *fr_box, decimation_factor=1)
    sim.run(until_after_sources=mp.stop_when_fields_decayed(50, mp.Ez, mp.Vector3(), 1e-6))
    assert mp.get_force_freqs(force) == [1.0]
    return {"force": mp.get_forces(force), "force_dec": mp.get_forces(force_dec),
            "force_box": mp.get_forces(force_box), "t": [sim.meep_time()]}


def _oracle_meep(oracle_lib):
    import os
    return os.path.join(os.path.dirname(oracle_lib), "liboracle_meep.so")


def test_python_script_on_oracle(oracle_lib):
    """add_force, get_forces and stop_when_fields_decayed in the Python front
    end (over the oracle) reproduce the reference core's run of the script:
    the same stop time, forces within 1e-13, and the reference test's golden
    master to 7 places."""
    out = script_force(_oracle_meep(oracle_lib))
    _check(out, golden("py_force", "f64"), 1e-13, 1e-13, False)
    assert round(out["force"][0] - REFERENCE_FORCE, 7) == 0


@pytest.mark.gpu
def test_gpu_fp64_matches_reference(gpu_drivers, tmp_path):
    """CUDA engine, FP64: fields bit-identical, forces within 1e-10."""
    _check(run_driver(GPU_DRIVER[64], "py_force", tmp_path), golden("py_force", "f64"), 1e-10, 1e-10, True)


@pytest.mark.gpu
def test_gpu_fp32_close_to_reference(gpu_drivers, tmp_path):
    """FP32 fields, FP64 DFT sums: forces within 1e-6 of the FP64 reference
    (the reference's own FP32 build: 5e-8)."""
    _check(run_driver(GPU_DRIVER[32], "py_force", tmp_path), golden("py_force", "f64"), 1e-6, 1e-6, False)


@pytest.mark.gpu
def test_gpu_python_script(gpu_drivers):
    """The Python script on the CUDA engine: the reference test's golden
    master to 7 places."""
    from meep_gb300.simulation import PRODUCT_LIB
    out = script_force(PRODUCT_LIB)
    _check(out, golden("py_force", "f64"), 1e-10, 1e-10, False)
    assert round(out["force"][0] - REFERENCE_FORCE, 7) == 0
