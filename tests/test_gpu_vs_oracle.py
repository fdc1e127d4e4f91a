"""GPU: the C ABI of the CUDA engine against the CPU oracle on the same seeded
random problems (random materials, conductivity, Drude/Lorentz poles,
integrated and current sources, DFT monitors), 2-D and 3-D, FP64 and FP32."""
import numpy as np
import pytest

from harness import random_problem, relerr
from meep_gb300 import _lib

pytestmark = pytest.mark.gpu


def _run(lib, seed, dim, prec, **kw):
    eng = _lib.Engine(lib)
    return random_problem(lambda **k: _lib.Sim(eng, **k), seed, dim, precision=prec, **kw)


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_fp64_bitwise_class(dim, seed, engine_lib, oracle_lib):
    g = _run(engine_lib, seed, dim, 64)
    o = _run(oracle_lib, seed, dim, 64)
    for k in o:
        assert relerr(g[k], o[k]) <= 1e-12, (k, relerr(g[k], o[k]))


@pytest.mark.parametrize("dim", [2, 3])
def test_fp32_close(dim, engine_lib, oracle_lib):
    g = _run(engine_lib, 7, dim, 32)
    o = _run(oracle_lib, 7, dim, 64)
    for k in o:
        assert relerr(g[k], o[k]) <= 1e-3, (k, relerr(g[k], o[k]))


# FP32 engine against the FP32 oracle (same arithmetic, rounding differs only
# by fused multiply-adds): a wrong branch at any PML, wall, conductivity or
# pole point shows up as an O(1) error.  The long-z grids span several warps
# of four-point quads along the unit-stride axis, with rows whose length is
# not a multiple of four.
@pytest.mark.parametrize("seed,n", [(11, None), (12, None), (13, (18, 16, 141)), (14, (16, 17, 262)),
                                    (15, (13, 11, 130))])
def test_fp32_matches_fp32_oracle(seed, n, engine_lib, oracle_lib):
    g = _run(engine_lib, seed, 3, 32, n=n)
    o = _run(oracle_lib, seed, 3, 32, n=n)
    for k in o:
        assert relerr(g[k], o[k]) <= 2e-5, (k, relerr(g[k], o[k]))


# Bloch-periodic boundaries with complex fields (and k = 0: real fields,
# periodic copies), PML in the other directions, dispersive and conductive
# media: same random problems on the GPU and the oracle
@pytest.mark.parametrize("dim,seed,bloch", [(2, 31, {0: 0.17}), (2, 32, {0: 0.0, 1: 0.23}),
                                            (3, 33, {0: 0.11, 2: 0.3}), (3, 34, {1: 0.0})])
def test_bloch_fp64_bitwise_class(dim, seed, bloch, engine_lib, oracle_lib):
    g = _run(engine_lib, seed, dim, 64, bloch=bloch)
    o = _run(oracle_lib, seed, dim, 64, bloch=bloch)
    for k in o:
        assert relerr(g[k], o[k]) <= 1e-12, (k, relerr(g[k], o[k]))


def test_bloch_with_pml_fp64_bitwise_class(engine_lib, oracle_lib):
    """periodic boundaries behind PML in the same direction (Simulation with
    k_point and PML layers)"""
    for dim, seed, bloch in ((2, 36, {0: 0.0, 1: 0.0}), (3, 37, {0: 0.15, 1: 0.0, 2: 0.05})):
        g = _run(engine_lib, seed, dim, 64, bloch=bloch, bloch_pml=True)
        o = _run(oracle_lib, seed, dim, 64, bloch=bloch, bloch_pml=True)
        for k in o:
            assert relerr(g[k], o[k]) <= 1e-12, (dim, k, relerr(g[k], o[k]))


def test_bloch_fp32_close(engine_lib, oracle_lib):
    g = _run(engine_lib, 35, 3, 32, bloch={0: 0.2, 1: 0.1})
    o = _run(oracle_lib, 35, 3, 64, bloch={0: 0.2, 1: 0.1})
    for k in o:
        assert relerr(g[k], o[k]) <= 1e-3, (k, relerr(g[k], o[k]))


@pytest.mark.parametrize("seed,poles,pml", [(41, True, True), (42, False, True), (43, True, False)])
def test_offdiag_3d_fp64_bitwise(seed, poles, pml, engine_lib, oracle_lib):
    """Off-diagonal inverse permittivity on the 3-D two-pass band kernels (D,
    f_minus_p; then E with OFFDIAG terms and poles): the same bits as the
    oracle's restatement of update_eh, with PML, poles and integrated sources."""
    kw = dict(poles=poles, pml=pml, offdiag=True, ecur=False, steps=50)
    out = random_problem(lambda **k: _lib.Sim(_lib.Engine(engine_lib), **k), seed, 3, **kw)
    ref = random_problem(lambda **k: _lib.Sim(_lib.Engine(oracle_lib), **k), seed, 3, **kw)
    for k in ref:
        if k.startswith("c"):
            assert np.array_equal(out[k], ref[k]), k
        else:
            assert relerr(out[k], ref[k]) <= 1e-13, k


def test_offdiag_3d_fp32_close(engine_lib, oracle_lib):
    kw = dict(offdiag=True, ecur=False, steps=50, precision=32)
    out = random_problem(lambda **k: _lib.Sim(_lib.Engine(engine_lib), **k), 44, 3, **kw)
    ref = random_problem(lambda **k: _lib.Sim(_lib.Engine(oracle_lib), **k), 44, 3, **kw)
    for k in ref:
        assert relerr(out[k], ref[k]) <= 1e-4, (k, relerr(out[k], ref[k]))


@pytest.mark.parametrize("seed,n,offdiag", [(51, (14, 12, 100), False), (52, (12, 13, 133), False),
                                            (53, (13, 12, 97), True)])
def test_boxed_materials_fp64_bitwise(seed, n, offdiag, engine_lib, oracle_lib):
    """Poles and conductivities present only inside boxes on grids with long
    z rows: the 3-D band kernels skip the pole and conductivity operands of
    row segments (32 z points) that hold none of them, which must leave every
    field bit unchanged (P stays 0 where sigma is 0)."""
    kw = dict(boxed=True, ecur=False, n=n, steps=60, offdiag=offdiag)
    g = _run(engine_lib, seed, 3, 64, **kw)
    o = _run(oracle_lib, seed, 3, 64, **kw)
    for k in o:
        if k.startswith("c"):
            assert np.array_equal(g[k], o[k]), k
        else:
            assert relerr(g[k], o[k]) <= 1e-13, (k, relerr(g[k], o[k]))


def test_boxed_materials_fp32(engine_lib, oracle_lib):
    kw = dict(boxed=True, ecur=False, n=(14, 12, 100), steps=60)
    g = _run(engine_lib, 54, 3, 32, **kw)
    o = _run(oracle_lib, 54, 3, 32, **kw)
    for k in o:
        assert relerr(g[k], o[k]) <= 2e-5, (k, relerr(g[k], o[k]))


@pytest.mark.parametrize("seed,n,boxed,offdiag", [(61, (18, 16, 100), False, False), (62, (17, 16, 97), True, False),
                                                  (63, (16, 18, 130), True, True), (64, (18, 16, 20), False, False)])
def test_palette_materials_fp64_bitwise(seed, n, boxed, offdiag, engine_lib, oracle_lib):
    """Materials from a few values (boxed and layered media as a structure
    built from objects has them), long z rows: every field bit of the 3-D
    band kernels equals the oracle's."""
    kw = dict(palette=True, boxed=boxed, ecur=False, n=n, steps=60, offdiag=offdiag)
    g = _run(engine_lib, seed, 3, 64, **kw)
    o = _run(oracle_lib, seed, 3, 64, **kw)
    for k in o:
        if k.startswith("c"):
            assert np.array_equal(g[k], o[k]), k
        else:
            assert relerr(g[k], o[k]) <= 1e-13, (k, relerr(g[k], o[k]))


def test_palette_materials_fp32(engine_lib, oracle_lib):
    kw = dict(palette=True, boxed=True, ecur=False, n=(18, 16, 100), steps=60)
    g = _run(engine_lib, 65, 3, 32, **kw)
    o = _run(oracle_lib, 65, 3, 32, **kw)
    for k in o:
        assert relerr(g[k], o[k]) <= 2e-5, (k, relerr(g[k], o[k]))


@pytest.mark.parametrize("seed,n,kw", [(71, (16, 14, 100), dict(bcond=True)),
                                       (72, (17, 15, 130), dict(poles_below=64)),
                                       (73, (16, 16, 100), dict(poles_below=48, bcond=True, palette=True))])
def test_bcond_and_layered_poles_fp64_bitwise(seed, n, kw, engine_lib, oracle_lib):
    """B conductivity (the B kernels' conductivity branch, FP32 quads on the
    faces) and poles confined to a low z layer (rows and faces split along z
    at the poles' extent): every field bit equals the oracle's in FP64."""
    kw = dict(kw, ecur=False, n=n, steps=60)
    g = _run(engine_lib, seed, 3, 64, **kw)
    o = _run(oracle_lib, seed, 3, 64, **kw)
    for k in o:
        if k.startswith("c"):
            assert np.array_equal(g[k], o[k]), k
        else:
            assert relerr(g[k], o[k]) <= 1e-13, (k, relerr(g[k], o[k]))


@pytest.mark.parametrize("seed,n,kw", [(71, (16, 14, 100), dict(bcond=True)),
                                       (72, (17, 15, 130), dict(poles_below=64)),
                                       (73, (16, 16, 100), dict(poles_below=48, bcond=True, palette=True))])
def test_bcond_and_layered_poles_fp32(seed, n, kw, engine_lib, oracle_lib):
    kw = dict(kw, ecur=False, n=n, steps=60)
    g = _run(engine_lib, seed, 3, 32, **kw)
    o = _run(oracle_lib, seed, 3, 32, **kw)
    for k in o:
        assert relerr(g[k], o[k]) <= 2e-5, (k, relerr(g[k], o[k]))


# the pole rows of the FP32 step take their activity word as a parameter when
# every segment there has the same one (poles on everywhere below z = 64, no
# conductivity): against the FP32 oracle, where a wrong bit shows as an O(1)
# error
@pytest.mark.parametrize("seed,n", [(75, (17, 15, 130)), (76, (18, 16, 100))])
def test_uniform_pole_layer_fp32(seed, n, engine_lib, oracle_lib):
    kw = dict(n=n, poles_below=64, cond=False, ecur=False, steps=60)
    g = _run(engine_lib, seed, 3, 32, **kw)
    o = _run(oracle_lib, seed, 3, 32, **kw)
    for k in o:
        assert relerr(g[k], o[k]) <= 2e-5, (k, relerr(g[k], o[k]))

