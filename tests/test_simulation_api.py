"""The Python Simulation front end (meep_gb300.Simulation) on scripts of the
reference's Python interface, against fixtures written by the reference core
for the same scripts (tests/golden/golden_driver.cpp, cases py_tm2d and
py_disp3d, which restate the C++ calls the reference's Python layer makes).

CPU: the front end over the meep:: drop-in on the CPU oracle.
GPU: the same over the CUDA engine (FP64 and FP32)."""
import os

import numpy as np
import pytest

from harness import golden, relerr
import meep_gb300 as mp
from meep_gb300.simulation import PRODUCT_LIB

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SINGLE_LIB = os.path.join(ROOT, "meep_gb300", "lib", "libmeep_gb300_single.so")


def script_tm2d(lib):
    geometry = [mp.Block(mp.Vector3(mp.inf, 1, mp.inf), material=mp.Medium(epsilon=12)),
                mp.Cylinder(0.8, center=mp.Vector3(3, 1.5), material=mp.Medium(index=2)),
                mp.Sphere(0.6, center=mp.Vector3(-2, -1.7), material=mp.Medium(epsilon=6, D_conductivity=0.05))]
    sim = mp.Simulation(cell_size=mp.Vector3(16, 8), resolution=10, geometry=geometry,
                        boundary_layers=[mp.PML(1.0)], eps_averaging=False,
                        sources=[mp.Source(mp.GaussianSource(0.15, fwidth=0.1), component=mp.Ez,
                                           center=mp.Vector3(-6), size=mp.Vector3(y=1))], _library=lib)
    tran = sim.add_flux([0.1, 0.125, 0.15, 0.175, 0.2], mp.FluxRegion(center=mp.Vector3(6), size=mp.Vector3(y=2)))
    box = sim.add_flux(0.15, 0.05, 3, mp.FluxRegion(center=mp.Vector3(4), size=mp.Vector3(y=3)),
                       mp.FluxRegion(center=mp.Vector3(2), size=mp.Vector3(y=3), weight=-1))
    dft = sim.add_dft_fields([mp.Ez], [0.12, 0.15], center=mp.Vector3(5), size=mp.Vector3(1, 2))
    sim.run(until_after_sources=30)
    return {"flux_tran": mp.get_fluxes(tran), "flux_box": mp.get_fluxes(box), "t": sim.meep_time(),
            "Ez": sim.get_yee_array(mp.Ez).reshape(-1), "Hy": sim.get_yee_array(mp.Hy).reshape(-1),
            "dft_Ez": [sim.get_dft_array(dft, mp.Ez, i) for i in range(2)]}


def script_disp3d(lib):
    mat = mp.Medium(epsilon=2, E_susceptibilities=[
        mp.LorentzianSusceptibility(frequency=1.1, gamma=0.1, sigma=0.5),
        mp.DrudeSusceptibility(frequency=0.8, gamma=0.05, sigma=0.3)])
    geometry = [mp.Block(mp.Vector3(1.2, 1.2, 1.2), material=mat),
                mp.Sphere(0.4, center=mp.Vector3(0.6), material=mp.Medium(epsilon_diag=mp.Vector3(2, 3, 4)))]
    sim = mp.Simulation(cell_size=mp.Vector3(3, 3, 3), resolution=10, geometry=geometry,
                        boundary_layers=[mp.PML(0.5)], eps_averaging=False,
                        sources=[mp.Source(mp.GaussianSource(0.8, fwidth=0.5, is_integrated=True), component=mp.Ex,
                                           center=mp.Vector3(-0.7, 0.1))], _library=lib)
    flux = sim.add_flux(0.8, 0.4, 4, mp.FluxRegion(center=mp.Vector3(z=0.9), size=mp.Vector3(2, 2)))
    sim.run(until=8)
    return {"flux": mp.get_fluxes(flux), "t": sim.meep_time(), "Ex": sim.get_yee_array(mp.Ex).reshape(-1),
            "Hy": sim.get_yee_array(mp.Hy).reshape(-1)}


def script_aniso_te2d(lib):
    """Default eps_averaging=True (subpixel averaging on the GPU), TE fields."""
    geometry = [mp.Block(mp.Vector3(mp.inf, 1, mp.inf), center=mp.Vector3(y=0.17), material=mp.Medium(epsilon=12)),
                mp.Cylinder(0.8, center=mp.Vector3(3, 1.5), material=mp.Medium(index=2)),
                mp.Sphere(0.6, center=mp.Vector3(-2, -1.7), material=mp.Medium(epsilon=6, D_conductivity=0.05))]
    sim = mp.Simulation(cell_size=mp.Vector3(16, 8), resolution=10, geometry=geometry,
                        boundary_layers=[mp.PML(1.0)],
                        sources=[mp.Source(mp.GaussianSource(0.15, fwidth=0.1), component=mp.Ey,
                                           center=mp.Vector3(-6), size=mp.Vector3(y=1))], _library=lib)
    tran = sim.add_flux([0.1, 0.15, 0.2], mp.FluxRegion(center=mp.Vector3(6), size=mp.Vector3(y=2)))
    sim.run(until_after_sources=20)
    return {"flux": mp.get_fluxes(tran), "t": sim.meep_time(), "Ex": sim.get_yee_array(mp.Ex).reshape(-1),
            "Ey": sim.get_yee_array(mp.Ey).reshape(-1), "Hz": sim.get_yee_array(mp.Hz).reshape(-1)}


def script_aniso3d(lib):
    mat = mp.Medium(epsilon=2.5, E_susceptibilities=[mp.LorentzianSusceptibility(frequency=1.1, gamma=0.1, sigma=0.5)])
    geometry = [mp.Block(mp.Vector3(1.1, 0.9, 0.73), center=mp.Vector3(0.05, -0.1, 0.02), material=mat),
                mp.Cylinder(0.35, height=1.0, axis=mp.Vector3(0.6, 0, 0.8), center=mp.Vector3(0.2, 0.3, -0.1),
                            material=mp.Medium(epsilon=5))]
    sim = mp.Simulation(cell_size=mp.Vector3(2, 2, 2), resolution=10, geometry=geometry,
                        boundary_layers=[mp.PML(0.5)],
                        sources=[mp.Source(mp.GaussianSource(0.8, fwidth=0.5, is_integrated=True), component=mp.Ex,
                                           center=mp.Vector3(-0.4, 0.1))], _library=lib)
    flux = sim.add_flux(0.8, 0.4, 3, mp.FluxRegion(center=mp.Vector3(z=0.45), size=mp.Vector3(1, 1)))
    sim.run(until=6)
    return {"flux": mp.get_fluxes(flux), "t": sim.meep_time(), "Ex": sim.get_yee_array(mp.Ex).reshape(-1),
            "Ez": sim.get_yee_array(mp.Ez).reshape(-1), "Hy": sim.get_yee_array(mp.Hy).reshape(-1)}


def _dft_from_fixture(rec, nd, nf):
    rows = np.asarray(rec).reshape(-1, nd + 2 * nf)
    return [rows[:, nd + 2 * w] + 1j * rows[:, nd + 2 * w + 1] for w in range(nf)]


def _compare(out, ref, tol):
    for k, v in ref.items():
        if k == "realnum_bytes" or k.startswith("chi_"):
            continue
        if k == "dft_Ez":
            for w, r in enumerate(_dft_from_fixture(v, 2, 2)):
                o = np.asarray(out[k][w]).reshape(-1)
                assert relerr(np.concatenate([o.real, o.imag]), np.concatenate([r.real, r.imag])) <= tol, (k, w)
            continue
        o = np.asarray(out[k], dtype=np.float64).reshape(-1)
        assert relerr(o, np.asarray(v).reshape(-1)) <= tol, (k, relerr(o, np.asarray(v).reshape(-1)))


@pytest.fixture(scope="module")
def oracle_meep_lib(oracle_lib):
    return os.path.join(os.path.dirname(oracle_lib), "liboracle_meep.so")


def test_script_tm2d_on_oracle(oracle_meep_lib):
    _compare(script_tm2d(oracle_meep_lib), golden("py_tm2d"), 1e-10)


def test_script_disp3d_on_oracle(oracle_meep_lib):
    _compare(script_disp3d(oracle_meep_lib), golden("py_disp3d"), 1e-10)


@pytest.mark.parametrize("script,case", [(script_aniso_te2d, "py_aniso_te2d"), (script_aniso3d, "py_aniso3d")])
def test_averaged_script_on_oracle(script, case, oracle_meep_lib):
    """eps_averaging=True: the averaged tensors (host evaluation of the same
    routine) and fields equal the reference core's averaging of the objects."""
    _compare(script(oracle_meep_lib), golden(case), 1e-10)


def test_run_until_step_count(oracle_meep_lib):
    """run(until=T) stops at the first step with round_time() >= T, as the
    reference's _run_until does; a second run continues from there."""
    sim = mp.Simulation(cell_size=mp.Vector3(4, 4), resolution=10, eps_averaging=False,
                        sources=[mp.Source(mp.ContinuousSource(0.5), component=mp.Ez, center=mp.Vector3())],
                        _library=oracle_meep_lib)
    sim.run(until=3)
    assert sim.timestep() == 60
    sim.run(until=0.26)
    assert sim.timestep() == 66
    calls = []
    sim.run(mp.at_every(0.5, lambda s: calls.append(s.meep_time())), until=2)
    assert sim.timestep() == 106 and len(calls) == 5


def test_unsupported_options_raise(oracle_meep_lib):
    with pytest.raises(NotImplementedError, match="eps_averaging"):
        mp.Simulation(cell_size=mp.Vector3(4, 4), resolution=10, _library=oracle_meep_lib,
                      geometry=[mp.Block(mp.Vector3(1, 1), material=mp.Medium(epsilon_diag=mp.Vector3(2, 3, 2)))])
    with pytest.raises(NotImplementedError, match="material functions"):
        mp.Block(mp.Vector3(1, 1), material=lambda p: mp.Medium(epsilon=2))


@pytest.mark.gpu
def test_script_tm2d_on_gpu(engine_lib):
    _compare(script_tm2d(PRODUCT_LIB), golden("py_tm2d"), 1e-10)


@pytest.mark.gpu
def test_script_disp3d_on_gpu(engine_lib):
    _compare(script_disp3d(PRODUCT_LIB), golden("py_disp3d"), 1e-10)


@pytest.mark.gpu
@pytest.mark.parametrize("script,case", [(script_aniso_te2d, "py_aniso_te2d"), (script_aniso3d, "py_aniso3d")])
def test_averaged_script_on_gpu(script, case, engine_lib):
    """eps_averaging=True with the averaging on the GPU (mfd_subpixel_rows):
    bit-identical to the reference core's averaging."""
    _compare(script(PRODUCT_LIB), golden(case), 1e-10)


@pytest.mark.gpu
def test_scripts_fp32_on_gpu(engine_lib):
    for script, case in ((script_tm2d, "py_tm2d"), (script_disp3d, "py_disp3d")):
        out = script(SINGLE_LIB)
        ref64, ref32 = golden(case), golden(case, "f32")
        for k in ("Ez", "Hy", "Ex", "flux", "flux_tran"):
            if k in ref64:
                bound = max(3 * relerr(ref32[k], ref64[k]), 1e-5)
                assert relerr(np.reshape(out[k], -1), ref64[k]) <= bound, (case, k)


def integrated_source_std(lib):
    """The reference's python/tests/test_integrated_source.py: an
    is_integrated=True line source extending into the PML of a periodic cell
    (k_point = 0) makes a planewave, so Ez on a parallel line is constant."""
    sources = [mp.Source(mp.ContinuousSource(1, is_integrated=True), center=mp.Vector3(-2), size=mp.Vector3(y=6),
                         component=mp.Ez)]
    sim = mp.Simulation(resolution=20, cell_size=(6, 6), boundary_layers=[mp.PML(thickness=1)], sources=sources,
                        k_point=mp.Vector3(), _library=lib)
    sim.run(until=30)
    ez = sim.get_array(mp.Ez, center=mp.Vector3(2), size=mp.Vector3(y=6))
    return np.std(ez) / np.sqrt(np.mean(ez ** 2))


def test_integrated_source_planewave_on_oracle(oracle_meep_lib):
    assert abs(integrated_source_std(oracle_meep_lib)) < 1e-8


@pytest.mark.gpu
def test_integrated_source_planewave_on_gpu(engine_lib):
    assert abs(integrated_source_std(PRODUCT_LIB)) < 1e-8


def test_precision_from_environment(monkeypatch):
    """MEEP_GB300_PRECISION picks the drop-in build Simulation loads (the
    reference picks realnum when it is built)."""
    from meep_gb300 import simulation as sm
    monkeypatch.delenv("MEEP_GB300_PRECISION", raising=False)
    assert sm._product_lib() == sm.DOUBLE_LIB
    monkeypatch.setenv("MEEP_GB300_PRECISION", "32")
    assert sm._product_lib() == sm.SINGLE_LIB
    monkeypatch.setenv("MEEP_GB300_PRECISION", "64")
    assert sm._product_lib() == sm.DOUBLE_LIB
    monkeypatch.setenv("MEEP_GB300_PRECISION", "16")
    with pytest.raises(ValueError):
        sm._product_lib()


# --- material grids ----------------------------------------------------------

def script_matgrid(lib, beta=6):
    """golden_driver case py_matgrid: a projected MaterialGrid block beside a
    cylinder (the weights come from the fixture)."""
    u = np.asarray(golden("py_matgrid")["weights"]).reshape(15, 11)
    mg = mp.MaterialGrid(mp.Vector3(15, 11), mp.Medium(epsilon=1.5), mp.Medium(epsilon=9), weights=u, beta=beta,
                         eta=0.45)
    geometry = [mp.Cylinder(0.6, center=mp.Vector3(-2, 1.5), material=mp.Medium(epsilon=4)),
                mp.Block(center=mp.Vector3(0.3, -0.2), size=mp.Vector3(3.1, 2.3), material=mg)]
    sim = mp.Simulation(cell_size=mp.Vector3(10, 8), resolution=10, geometry=geometry,
                        boundary_layers=[mp.PML(1.0)], eps_averaging=False,
                        sources=[mp.Source(mp.GaussianSource(0.2, fwidth=0.2), component=mp.Ez,
                                           center=mp.Vector3(-3, 0))], _library=lib)
    flux = sim.add_flux(0.2, 0.2, 5, mp.FluxRegion(center=mp.Vector3(3), size=mp.Vector3(0, 4)))
    sim.run(until=60)
    return {"flux": mp.get_fluxes(flux), "t": sim.meep_time(), "Ez": sim.get_yee_array(mp.Ez).reshape(-1),
            "weights": u.reshape(-1)}


def test_script_matgrid_on_oracle(oracle_meep_lib):
    """MaterialGrid through the front end, evaluated by the CPU oracle: within
    1e-12 of the reference core running the restated grid material (the
    projection's tanh and the points' coordinates may round differently)."""
    _compare(script_matgrid(oracle_meep_lib), golden("py_matgrid"), 1e-12)


def test_matgrid_unsupported_options_raise(oracle_meep_lib):
    m1, m2 = mp.Medium(epsilon=1), mp.Medium(epsilon=4)
    with pytest.raises(NotImplementedError, match="smoothing"):
        mp.MaterialGrid(mp.Vector3(3, 3), m1, m2, do_averaging=True)
    with pytest.raises(NotImplementedError, match="U_MEAN"):
        mp.MaterialGrid(mp.Vector3(3, 3), m1, m2, grid_type="U_MEAN")
    with pytest.raises(NotImplementedError, match="dispersive"):
        mp.MaterialGrid(mp.Vector3(3, 3), m1, mp.Medium(epsilon=2, D_conductivity=0.1))
    with pytest.raises(ValueError):
        mp.MaterialGrid(mp.Vector3(3, 3), m1, m2, weights=np.zeros(4))
    with pytest.warns(UserWarning, match="range"):
        g = mp.MaterialGrid(mp.Vector3(2, 2), m1, m2, weights=np.array([-0.5, 0.2, 0.7, 1.5]))
    assert list(g.weights) == [0.0, 0.2, 0.7, 1.0]
    sim = mp.Simulation(cell_size=mp.Vector3(4, 4), resolution=10, default_material=g, _library=oracle_meep_lib,
                        sources=[mp.Source(mp.GaussianSource(0.2, fwidth=0.2), component=mp.Ez,
                                           center=mp.Vector3())])
    with pytest.raises(NotImplementedError, match="default material"):
        sim.init_sim()
    sim = mp.Simulation(cell_size=mp.Vector3(4, 4), resolution=10, _library=oracle_meep_lib,
                        geometry=[mp.Sphere(0.5, material=g)],
                        sources=[mp.Source(mp.GaussianSource(0.2, fwidth=0.2), component=mp.Ez,
                                           center=mp.Vector3())])
    with pytest.raises(NotImplementedError, match="Block"):
        sim.init_sim()


@pytest.mark.gpu
def test_script_matgrid_on_gpu(engine_lib):
    """The same on the CUDA engine (grid evaluated on the device): FP64
    within 1e-12 of the reference core, FP32 within 3x the reference's own
    FP32 error (or 1e-5)."""
    _compare(script_matgrid(PRODUCT_LIB), golden("py_matgrid"), 1e-12)
    out = script_matgrid(SINGLE_LIB)
    ref64, ref32 = golden("py_matgrid"), golden("py_matgrid", "f32")
    for k in ("Ez", "flux"):
        bound = max(3 * relerr(ref32[k], ref64[k]), 1e-5)
        assert relerr(np.reshape(out[k], -1), ref64[k]) <= bound, k
