"""GPU: the reverse-time adjoint (exact discrete adjoint of the leapfrog step,
with PML) against central finite differences of the same time-stepped
objective, in FP64; record mode and sqrt(T)-checkpoint mode; FP32 adjoint
against the FP64 gradient."""
import numpy as np
import pytest

from harness import relerr, tm2d_design_problem
from meep_gb300 import _lib

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def design():
    rng = np.random.default_rng(11)
    return rng.uniform(1.0, 12.0, size=(12, 12))


def test_adjoint_matches_finite_differences(design, engine_lib):
    eng = _lib.Engine(engine_lib)
    J0, g = tm2d_design_problem(eng, design, precision=64)
    assert J0 > 0
    rng = np.random.default_rng(5)
    pix = [tuple(rng.integers(0, 12, size=2)) for _ in range(8)]
    h = 1e-4
    fd = []
    for (a, b) in pix:
        ep = design.copy()
        ep[a, b] += h
        em = design.copy()
        em[a, b] -= h
        Jp, _ = tm2d_design_problem(eng, ep, grad=False)
        Jm, _ = tm2d_design_problem(eng, em, grad=False)
        fd.append((Jp - Jm) / (2 * h))
    adj = np.array([g[a, b] for (a, b) in pix])
    fd = np.array(fd)
    assert relerr(adj, fd) <= 1e-4, (adj, fd)


def test_checkpointed_adjoint_equals_recorded(design, engine_lib):
    eng = _lib.Engine(engine_lib)
    _, g_rec = tm2d_design_problem(eng, design, precision=64, checkpoint_every=0)
    _, g_ck = tm2d_design_problem(eng, design, precision=64, checkpoint_every=25)
    assert relerr(g_ck, g_rec) <= 1e-12


def test_fp32_adjoint_close_to_fp64(design, engine_lib):
    eng = _lib.Engine(engine_lib)
    _, g64 = tm2d_design_problem(eng, design, precision=64)
    _, g32 = tm2d_design_problem(eng, design, precision=32)
    assert relerr(g32, g64) <= 1e-3
