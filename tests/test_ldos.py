"""Local density of states (dft_ldos, src/dft_ldos.cpp).

Case py_ldos of tests/golden/golden_driver.cpp: a 2-D off-grid Ez dipole
(four interpolation points) beside a dielectric block, the dft_ldos step
function at 5 frequencies, run 20 time units after the sources.  Records the
LDOS spectrum and the DFTs F (of E.J*) and J (of the source current)."""
import os

import numpy as np
import pytest

from harness import GPU_DRIVER, ORACLE_DRIVER, golden, run_driver


def _c(rec):
    a = np.asarray(rec)
    return a[0::2] + 1j * a[1::2]


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / np.abs(b).max())


def _check(out, ref, tol):
    assert out["t"][0] == ref["t"][0]
    assert _rel(out["ldos"], ref["ldos"]) <= tol
    assert _rel(_c(out["F"]), _c(ref["F"])) <= tol
    assert _rel(_c(out["J"]), _c(ref["J"])) <= tol


def test_oracle_fp64_matches_reference(oracle_lib, tmp_path):
    """The drop-in's dft_ldos over the CPU oracle: the same spectrum as the
    reference core within 1e-11 (F and J agree to 1e-14; the LDOS divides by
    |J|^2)."""
    _check(run_driver(ORACLE_DRIVER[64], "py_ldos", tmp_path), golden("py_ldos", "f64"), 1e-11)


def script_ldos(lib):
    import meep_gb300 as mp
    sim = mp.Simulation(cell_size=mp.Vector3(6, 6), resolution=20, boundary_layers=[mp.PML(1)], eps_averaging=False,
                        geometry=[mp.Block(mp.Vector3(1, 1, mp.inf), center=mp.Vector3(0.8),
                                           material=mp.Medium(epsilon=4))],
                        sources=[mp.Source(mp.GaussianSource(1.0, fwidth=0.2), component=mp.Ez,
                                           center=mp.Vector3(0.1, 0.05))], _library=lib)
    ldos = mp.Ldos(1.0, 0.2, 5)
    sim.run(mp.dft_ldos(ldos=ldos), until_after_sources=20)
    assert len(mp.get_ldos_freqs(ldos)) == 5
    ri = lambda v: list(np.stack([np.real(v), np.imag(v)], -1).ravel())
    return {"ldos": sim.ldos_data, "F": ri(sim.ldos_Fdata), "J": ri(sim.ldos_Jdata), "t": [sim.meep_time()]}


def test_python_script_on_oracle(oracle_lib):
    """mp.dft_ldos as a step function in the Python front end: the same
    spectrum as the reference core's run of the script."""
    _check(script_ldos(os.path.join(os.path.dirname(oracle_lib), "liboracle_meep.so")), golden("py_ldos", "f64"),
           1e-11)


@pytest.mark.gpu
def test_gpu_matches_reference(gpu_drivers, tmp_path):
    """CUDA engine: FP64 within 1e-10 of the reference, FP32 within 1e-4, and
    the Python script on the GPU within 1e-10."""
    ref = golden("py_ldos", "f64")
    _check(run_driver(GPU_DRIVER[64], "py_ldos", tmp_path), ref, 1e-10)
    _check(run_driver(GPU_DRIVER[32], "py_ldos", tmp_path), ref, 1e-4)
    from meep_gb300.simulation import PRODUCT_LIB
    _check(script_ldos(PRODUCT_LIB), ref, 1e-10)


def test_ldos_update_must_run_every_step(oracle_lib):
    """The engine's DFT of the fields samples every step, so an LDOS whose
    update runs less often (at_every) would mix samples: the results raise."""
    import meep_gb300 as mp
    lib = os.path.join(os.path.dirname(oracle_lib), "liboracle_meep.so")
    sim = mp.Simulation(cell_size=mp.Vector3(4, 4), resolution=10, boundary_layers=[mp.PML(1)], eps_averaging=False,
                        sources=[mp.Source(mp.GaussianSource(1.0, fwidth=0.2), component=mp.Ez,
                                           center=mp.Vector3())], _library=lib)
    ldos = mp.Ldos(1.0, 0.2, 3)
    with pytest.raises(RuntimeError, match="every step"):
        sim.run(mp.at_every(0.5, mp.dft_ldos(ldos=ldos)), until=5)
