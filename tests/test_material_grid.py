"""Material grids (mfd_add_material_grid / mfd_material_grid_vjp): the
projected, interpolated design weights as the diagonal inverse permittivity of
the E components inside a block, and dJ/du through the projection and the
interpolation.

The checker is a plain-Python restatement of the reference's formulas
(linear_interpolate with mirror faces, src/fields.cpp:759-806;
tanh_projection, src/meepgeom.cpp:497-502; epsilon_material_grid's
eps1 + u (eps2 - eps1), :569-581): the same problem stepped with the
restated chi1inv set point by point must give the same fields, and dJ/du must
meet central differences of J(u) = sum gchi * chi1inv(u)."""
import math

import numpy as np
import pytest

from harness import relerr
from meep_gb300 import _lib

NX, NY, RES = 40, 30, 10.0
CENTER, SIZE = (0.05, -0.1, 0.0), (1.6, 1.2, 0.0)
EPS1, EPS2 = (1.0, 1.5, 2.0), (12.0, 9.0, 6.0)


def _mirror(i, n):
    return 2 * n - 1 - i if i >= n else (-1 - i if i < 0 else i)


def _map(r, n):
    r = -r if r < 0.0 else (1.0 - r if r > 1.0 else r)
    i1 = _mirror(int(r * n), n)
    d = r * n - i1 - 0.5
    return i1, _mirror(i1 + 1 if d >= 0.0 else i1 - 1, n), abs(d)


def _interp(u, r):
    n = u.shape
    (x1, x2, dx), (y1, y2, dy), (z1, z2, dz) = (_map(r[d], n[d]) for d in range(3))
    U = lambda x, y, z: u[x, y, z]  # noqa: E731
    return (((U(x1, y1, z1) * (1.0 - dx) + U(x2, y1, z1) * dx) * (1.0 - dy) +
             (U(x1, y2, z1) * (1.0 - dx) + U(x2, y2, z1) * dx) * dy) * (1.0 - dz) +
            ((U(x1, y1, z2) * (1.0 - dx) + U(x2, y1, z2) * dx) * (1.0 - dy) +
             (U(x1, y2, z2) * (1.0 - dx) + U(x2, y2, z2) * dx) * dy) * dz)


def _project(u, beta, eta):
    if beta == 0:
        return u
    if u == eta:
        return 0.5
    t = math.tanh(beta * eta)
    return (t + math.tanh(beta * (u - eta))) / (t + math.tanh(beta * (1 - eta)))


def _chi_points(u, beta, eta, comp_dir, shift):
    """{(i, j): chi1inv} of the 2-D component with Yee shift `shift` (half
    pixels) along direction comp_dir, at the points inside the block."""
    out = {}
    for i in range(NX + 1):
        for j in range(NY + 1):
            x = ((-NX + shift[0] + 2 * i) * (0.5 * (1.0 / RES)), (-NY + shift[1] + 2 * j) * (0.5 * (1.0 / RES)), 0.0)
            if not all(abs(x[d] - CENTER[d]) <= 0.5 * SIZE[d] for d in range(3)):
                continue
            r = [0.0 if SIZE[d] == 0 else 0.5 + (x[d] - CENTER[d]) / SIZE[d] for d in range(3)]
            p = _project(_interp(u, r), beta, eta)
            out[(i, j)] = 1.0 / (EPS1[comp_dir] + p * (EPS2[comp_dir] - EPS1[comp_dir]))
    return out


def _weights(seed=3, n=(13, 9, 1)):
    return np.random.default_rng(seed).uniform(0.0, 1.0, size=n)


TE = ("TE", [(_lib.E, _lib.X), (_lib.E, _lib.Y), (_lib.H, _lib.Z), (_lib.D, _lib.X), (_lib.D, _lib.Y),
             (_lib.B, _lib.Z)], _lib.comp(_lib.E, _lib.Y))
TM = ("TM", [(_lib.E, _lib.Z), (_lib.H, _lib.X), (_lib.H, _lib.Y), (_lib.D, _lib.Z), (_lib.B, _lib.X),
             (_lib.B, _lib.Y)], _lib.comp(_lib.E, _lib.Z))
SHIFT = {_lib.X: (1, 0), _lib.Y: (0, 1), _lib.Z: (0, 0)}


def _sim(eng, pol, precision, u=None, beta=0.0, eta=0.5, restated=False):
    _, comps, src_c = pol
    cs = [_lib.comp(t, d) for t, d in comps]
    pml = {(d, s): (0.6, 1e-15, 1.0) for d in (0, 1) for s in (0, 1)}
    sim = _lib.Sim(eng, dim=2, n=(NX, NY, 0), io=(-NX, -NY, 0), a=RES, courant=0.5, pml=pml, precision=precision,
                   components=cs)
    ecomps = [_lib.comp(t, d) for t, d in comps if t == _lib.E]
    for c in ecomps:
        d = c % 3
        chi = np.full((NX + 1, NY + 1), 1.0 / 2.25)
        if restated:
            for (i, j), v in _chi_points(u, beta, eta, d, SHIFT[d]).items():
                chi[i, j] = v
        sim.set_chi1inv(c, d, chi)
    grid = None
    if u is not None and not restated:
        # the background 2.25 everywhere, the grid over the block
        grid = sim.add_material_grid(CENTER, SIZE, u, EPS1, EPS2, beta=beta, eta=eta)
    s = sim.add_gaussian_src(0.8, 0.4, integrated=True)
    sim.add_source_points(src_c, s, [(NX // 2 - 5) * (NY + 1) + NY // 2 + 2], [1.0])
    return sim, grid, ecomps


def _fields(sim, ecomps, steps):
    sim.step(steps)
    return np.concatenate([sim.get_field(c).reshape(-1) for c in ecomps])


@pytest.mark.parametrize("pol", [TM, TE], ids=["TM", "TE"])
@pytest.mark.parametrize("beta,eta", [(0.0, 0.5), (8.0, 0.4)])
def test_oracle_grid_equals_restated_chi(oracle_lib, pol, beta, eta):
    """CPU oracle: a material grid over a block gives the fields of the
    restated chi1inv set point by point (bit-identical without projection;
    within 1e-13 with it: the restatement's tanh is Python's)."""
    eng = _lib.Engine(oracle_lib)
    u = _weights()
    a, _, ec = _sim(eng, pol, 64, u, beta, eta)
    b, _, _ = _sim(eng, pol, 64, u, beta, eta, restated=True)
    fa, fb = _fields(a, ec, 60), _fields(b, ec, 60)
    a.close()
    b.close()
    assert np.abs(fa).max() > 0
    if beta == 0.0:
        assert np.array_equal(fa, fb)
    else:
        assert relerr(fa, fb) <= 1e-13


def _vjp_case(eng, pol, beta, eta, precision=64, seed=7):
    u = _weights()
    sim, grid, ec = _sim(eng, pol, precision, u, beta, eta)
    lo, hi = (10, 8, 0), (32, 22, 0)
    rng = np.random.default_rng(seed)
    box = (hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1)
    gchi = rng.standard_normal(len(ec) * box)
    gu = sim.material_grid_vjp(grid, gchi, comps=ec, lo=lo, hi=hi)
    sim.close()
    return u, ec, lo, hi, gchi, gu


def _J(u, ec, lo, hi, gchi, beta, eta):
    J, q = 0.0, 0
    for c in ec:
        d = c % 3
        chi = _chi_points(u, beta, eta, d, SHIFT[d])
        for i in range(lo[0], hi[0] + 1):
            for j in range(lo[1], hi[1] + 1):
                J += gchi[q] * chi.get((i, j), 0.0)
                q += 1
    return J


@pytest.mark.parametrize("pol", [TM, TE], ids=["TM", "TE"])
@pytest.mark.parametrize("beta,eta", [(0.0, 0.5), (8.0, 0.4)])
def test_oracle_vjp_matches_finite_differences(oracle_lib, pol, beta, eta):
    """dJ/du for J = sum gchi * chi1inv(u) over a box that holds the block and
    points outside it: central differences (h = 1e-6) of the restated J at
    twelve nodes, corners and faces included, within 1e-7."""
    eng = _lib.Engine(oracle_lib)
    u, ec, lo, hi, gchi, gu = _vjp_case(eng, pol, beta, eta)
    nodes = [(0, 0, 0), (12, 8, 0), (0, 8, 0), (12, 0, 0), (6, 4, 0), (1, 7, 0), (11, 1, 0), (3, 3, 0),
             (9, 5, 0), (5, 0, 0), (0, 5, 0), (12, 6, 0)]
    h = 1e-6
    fd = []
    for n in nodes:
        up, um = u.copy(), u.copy()
        up[n] += h
        um[n] -= h
        fd.append((_J(up, ec, lo, hi, gchi, beta, eta) - _J(um, ec, lo, hi, gchi, beta, eta)) / (2 * h))
    got = np.array([gu[n] for n in nodes])
    assert relerr(got, np.array(fd)) <= 1e-7, (got, fd)


def test_grid_argument_errors(oracle_lib):
    eng = _lib.Engine(oracle_lib)
    u = _weights()
    sim, _, ec = _sim(eng, TM, 64)
    with pytest.raises(_lib.MeepError, match="range"):
        sim.add_material_grid(CENTER, SIZE, u * 2, EPS1, EPS2)
    with pytest.raises(_lib.MeepError, match="eta"):
        sim.add_material_grid(CENTER, SIZE, u, EPS1, EPS2, beta=1.0, eta=1.5)
    with pytest.raises(_lib.MeepError, match="positive"):
        sim.add_material_grid(CENTER, SIZE, u, (0.0, 1.0, 1.0), EPS2)
    g = sim.add_material_grid(CENTER, SIZE, u, EPS1, EPS2)
    with pytest.raises(_lib.MeepError, match="out of range"):
        sim.material_grid_vjp(g + 1, np.zeros(4), comps=ec, lo=(0, 0, 0), hi=(1, 1, 0))
    with pytest.raises(_lib.MeepError, match="box"):
        sim.material_grid_vjp(g, np.zeros(4), comps=ec, lo=(0, 0, 0), hi=(NX + 1, 1, 0))
    sim.step(1)
    with pytest.raises(_lib.MeepError, match="before the first step"):
        sim.add_material_grid(CENTER, SIZE, u, EPS1, EPS2)
    sim.close()


@pytest.mark.gpu
@pytest.mark.parametrize("pol", [TM, TE], ids=["TM", "TE"])
@pytest.mark.parametrize("beta,eta", [(0.0, 0.5), (8.0, 0.4)])
def test_gpu_grid_matches_oracle(engine_lib, oracle_lib, pol, beta, eta):
    """CUDA engine: the device-evaluated grid gives the oracle's fields (FP64:
    bit-identical without projection, within 1e-12 with it, the device tanh
    differing from the host's in the last bits; FP32 within 1e-5), and the
    device dJ/du equals the host's within 1e-12."""
    gpu, cpu = _lib.Engine(engine_lib), _lib.Engine(oracle_lib)
    u = _weights()
    for prec, tol in ((64, 0.0 if beta == 0.0 else 1e-12), (32, 1e-5)):
        a, _, ec = _sim(gpu, pol, prec, u, beta, eta)
        b, _, _ = _sim(cpu, pol, prec, u, beta, eta)
        fa, fb = _fields(a, ec, 60), _fields(b, ec, 60)
        a.close()
        b.close()
        assert relerr(fa, fb) <= tol, (prec, relerr(fa, fb))
    _, _, _, _, _, g_gpu = _vjp_case(gpu, pol, beta, eta)
    _, _, _, _, _, g_cpu = _vjp_case(cpu, pol, beta, eta)
    assert relerr(g_gpu, g_cpu) <= 1e-12


@pytest.mark.gpu
def test_gpu_design_gradient_through_grid(engine_lib):
    """Reverse-time adjoint through a projected material grid (beta 8): dJ/du
    from mfd_backward + mfd_material_grid_vjp against central differences of
    the time-stepped J at six nodes (FP64, h = 1e-5), within 1e-6."""
    from meep_gb300.design import DesignProblem2D
    prob = DesignProblem2D(nx=120, ny=80, res=10.0, dpml_cells=10, guide_cells=6, design=(30, 30), nfreq=3,
                           line_cells=12, steps=700)
    grid = dict(n=(12, 12), eps1=1.5, eps2=10.0, beta=8.0, eta=0.5)
    u = np.random.default_rng(4).uniform(0.2, 0.8, size=(12, 12))
    F, handle = prob.run_grid(u, grid, grad=True)
    J0, dJdF = prob.objective(F)
    g = prob.backward_grid(handle, dJdF)
    h = 1e-5
    for n in [(0, 0), (11, 11), (5, 6), (2, 9), (8, 3), (6, 0)]:
        up, um = u.copy(), u.copy()
        up[n] += h
        um[n] -= h
        Jp = prob.objective(prob.run_grid(up, grid)[0])[0]
        Jm = prob.objective(prob.run_grid(um, grid)[0])[0]
        fd = (Jp - Jm) / (2 * h)
        assert abs(g[n] - fd) <= 1e-6 * np.abs(g).max(), (n, g[n], fd)
