"""The engine's reverse-time design gradient against the reference's
adjoint-solver gradient.

Fixture: tests/golden/adjoint_tm2d.f64.bin, written by the reference core
(oracle/ref/Makefile) running tests/golden/golden_driver.cpp case
adjoint_tm2d: a 2-D TM problem (100 x 60 pixels, PML, an eps = 12 guide, a
20 x 20-pixel design block with eps = eps1 + u (eps2 - eps1)), J = sum |F|^2
of the Ez DFT at f = 0.15 on an output line.  The reference runs the forward,
places the adjoint sources as its Python adjoint layer does
(python/adjoint/objective.py:65-153, 370-416: fourier_sourcedata amplitudes
of dJ = 2 conj(F) times _adj_src_scale), runs the adjoint and forms
dJ/du by material_grids_addgradient (src/meepgeom.cpp:2835-3011) for a pixel
material grid.  It also holds central differences of J on the reference core
at four pixels and along a random direction dp: the reference's adjoint
gradient agrees with them to 2.5e-6 (its own test asks 0.002 of the
directional derivative, python/tests/test_adjoint_solver.py:550).

The engine's gradient is the exact adjoint of the time-stepped objective
(mfd_forward / mfd_backward), so it must meet the reference's finite
differences and the reference's adjoint gradient at the level those two meet
each other."""
import numpy as np
import pytest

from harness import golden, relerr
from meep_gb300 import _lib

NX, NY, RES = 100, 60, 10.0
F0 = 0.15


def _fixture():
    return golden("adjoint_tm2d", "f64")


def _problem(eng, rec, precision, design=False):
    """The fixture's problem on an engine (C ABI): permittivity at the Ez
    points, the reference's source points and amplitudes, the objective line's
    Ez DFT with the reference's scale dt / sqrt(2 pi).  Returns (sim, monitor)."""
    ez = _lib.comp(_lib.E, _lib.Z)
    comps = [ez, _lib.comp(_lib.D, _lib.Z), _lib.comp(_lib.H, _lib.X), _lib.comp(_lib.B, _lib.X),
             _lib.comp(_lib.H, _lib.Y), _lib.comp(_lib.B, _lib.Y)]
    pml = {(d, s): (1.0, 1e-15, 1.0) for d in (0, 1) for s in (0, 1)}
    sim = _lib.Sim(eng, dim=2, n=(NX, NY, 0), io=(-NX, -NY, 0), a=RES, courant=0.5, pml=pml,
                   precision=precision, components=comps)
    eps = np.asarray(rec["eps"]).reshape(NX + 1, NY + 1)
    sim.set_chi1inv(ez, _lib.Z, 1.0 / eps)
    width = 1 / 0.1
    src = sim.add_gaussian_src(F0, width, integrated=False, window=(0.0, 2 * width * 5.0))
    sp = np.asarray(rec["src_points"]).reshape(-1, 4)
    idx = ((sp[:, 0] + NX) // 2).astype(np.int64) * (NY + 1) + ((sp[:, 1] + NY) // 2).astype(np.int64)
    sim.add_source_points(ez, src, idx, sp[:, 2] + 1j * sp[:, 3])
    F = np.asarray(rec["obj_F"]).reshape(-1, 4)
    i = int((F[0, 0] + NX) // 2)
    j0, j1 = int((F[:, 1].min() + NY) // 2), int((F[:, 1].max() + NY) // 2)
    assert (F[:, 0] == F[0, 0]).all() and j1 - j0 + 1 == len(F)
    dt = 0.5 / RES
    mid = sim.add_dft(ez, (i, j0, 0), (i, j1, 0), [np.ones(1), np.ones(j1 - j0 + 1), None], dV=1.0,
                      include_weights=False, scale=dt / np.sqrt(2 * np.pi), centered=False, freqs=[F0],
                      decimation=1)
    if design:
        lo_n = np.asarray(rec["design_lo_n"]).astype(int)
        lo = (lo_n[0], lo_n[1], 0)
        sim.design([ez], lo, (lo[0] + lo_n[2] - 1, lo[1] + lo_n[2] - 1, 0))
    return sim, mid


def _reference_F(rec):
    F = np.asarray(rec["obj_F"]).reshape(-1, 4)
    F = F[np.argsort(F[:, 1])]
    return F[:, 2] + 1j * F[:, 3]


def _engine_gradient(eng, rec, precision, checkpoint_every=100):
    """(F, dJ/du) of the engine: J = sum |F|^2, so dJ/dRe F + i dJ/dIm F = 2 F;
    dJ/du = dJ/deps (eps2 - eps1) with dJ/deps = -dJ/dchi1inv / eps^2."""
    steps = int(np.asarray(rec["steps"])[0])
    sim, mid = _problem(eng, rec, precision, design=True)
    try:
        sim.forward(steps, checkpoint_every)
        F = sim.get_dft(mid)[:, 0]
        gchi = sim.backward({mid: (2.0 * F)[:, None]})[0, :, :, 0]
    finally:
        sim.close()
    lo_n = np.asarray(rec["design_lo_n"]).astype(int)
    eps = np.asarray(rec["eps"]).reshape(NX + 1, NY + 1)
    e = eps[lo_n[0]:lo_n[0] + lo_n[2], lo_n[1]:lo_n[1] + lo_n[2]]
    e1, e2 = np.asarray(rec["eps12"])
    return F, (-gchi / (e * e) * (e2 - e1)).reshape(-1)


def test_fixture_pins_reference_gradient():
    """The reference's adjoint gradient against its own central differences
    (J on the reference core, u +- 1e-3): within 1e-5 at the four pixels of
    largest gradient and along the random direction."""
    rec = _fixture()
    g = np.asarray(rec["grad_u"])
    fd = np.asarray(rec["fd_pixels"]).reshape(-1, 2)
    k = fd[:, 0].astype(int)
    assert relerr(g[k], fd[:, 1]) <= 1e-5, (g[k], fd[:, 1])
    dd = float(np.asarray(rec["dp"]) @ g)
    assert abs(dd / float(np.asarray(rec["fd_directional"])[0]) - 1) <= 1e-5


def test_problem_matches_reference_on_oracle(oracle_lib):
    """The problem built through the C ABI is the reference's: on the CPU
    oracle the forward DFT on the objective line equals the reference core's
    within 1e-11 after the full forward run."""
    rec = _fixture()
    eng = _lib.Engine(oracle_lib)
    sim, mid = _problem(eng, rec, 64)
    try:
        sim.step(int(np.asarray(rec["steps"])[0]))
        F = sim.get_dft(mid)[:, 0]
    finally:
        sim.close()
    assert relerr(F, _reference_F(rec)) <= 1e-11, relerr(F, _reference_F(rec))


@pytest.mark.gpu
def test_gradient_matches_reference_adjoint_fp64(engine_lib):
    """FP64 engine, sqrt(T)-style checkpoints every 100 steps: the forward DFT
    within 1e-10 of the reference's; dJ/du within 1e-5 (relative, infinity
    norm over the 400 pixels) of the reference's adjoint-solver gradient and of
    its finite differences at four pixels; the directional derivative along dp
    within 1e-5 of both.  The reference's gradient is a frequency-domain
    estimate: it meets its own finite differences within 2.5e-6 at the
    largest pixels, and the engine's exact gradient within 7.3e-6 over all
    pixels (measured); 1e-5 is 200x tighter than the reference test's 0.002."""
    rec = _fixture()
    eng = _lib.Engine(engine_lib)
    F, g = _engine_gradient(eng, rec, 64)
    assert relerr(F, _reference_F(rec)) <= 1e-10, relerr(F, _reference_F(rec))
    gm = np.asarray(rec["grad_u"])
    print("FP64 engine vs reference adjoint gradient: %.3g" % relerr(g, gm))
    assert relerr(g, gm) <= 1e-5, relerr(g, gm)
    fd = np.asarray(rec["fd_pixels"]).reshape(-1, 2)
    assert relerr(g[fd[:, 0].astype(int)], fd[:, 1]) <= 1e-5
    dp = np.asarray(rec["dp"])
    fdd = float(np.asarray(rec["fd_directional"])[0])
    assert abs(dp @ g / fdd - 1) <= 1e-5 and abs(dp @ g / (dp @ gm) - 1) <= 1e-5


@pytest.mark.gpu
def test_gradient_matches_reference_adjoint_fp32(engine_lib):
    """FP32 engine (fields, adjoint fields and their products in single
    precision, DFT sums in double): dJ/du within 5e-5 of the reference's FP64
    adjoint-solver gradient (measured 7.8e-6), the directional derivative
    within 5e-5 (the reference test allows 0.075 for its FP32 build,
    python/tests/test_adjoint_solver.py:550)."""
    rec = _fixture()
    eng = _lib.Engine(engine_lib)
    F, g = _engine_gradient(eng, rec, 32)
    assert relerr(F, _reference_F(rec)) <= 1e-4
    gm = np.asarray(rec["grad_u"])
    print("FP32 engine vs reference adjoint gradient: %.3g" % relerr(g, gm))
    assert relerr(g, gm) <= 5e-5, relerr(g, gm)
    dp = np.asarray(rec["dp"])
    assert abs(dp @ g / (dp @ gm) - 1) <= 5e-5
