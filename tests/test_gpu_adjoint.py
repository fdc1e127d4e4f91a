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


def test_design_problem_full_size_vs_fd(engine_lib):
    """400x240 cells, 16-cell PML, 100x100 design block (eps uniform in [1,12]
    from a seed), 10 frequencies on a 20-cell output line, 3000 steps,
    checkpoints every 55 steps: adjoint gradient vs central finite differences
    (h = 1e-4, FP64) at 20 random design pixels."""
    from meep_gb300.design import DesignProblem2D

    prob = DesignProblem2D(_lib.Engine(engine_lib))
    rng = np.random.default_rng(2024)
    eps = rng.uniform(1.0, 12.0, size=prob.design)
    F, handle = prob.run(eps, grad=True, checkpoint_every=55)
    J, dJdF = prob.objective(F)
    g = prob.backward(handle, dJdF)
    pix = [tuple(rng.integers(0, prob.design[0], size=2)) for _ in range(20)]
    h = 1e-4
    fd = []
    for (a, b) in pix:
        ep = eps.copy()
        ep[a, b] += h
        em = eps.copy()
        em[a, b] -= h
        fd.append((prob.objective(prob.run(ep)[0])[0] - prob.objective(prob.run(em)[0])[0]) / (2 * h))
    adj = np.array([g[a, b] for (a, b) in pix])
    assert relerr(adj, np.array(fd)) <= 1e-4


def test_torch_autograd_wrapper(engine_lib):
    torch = pytest.importorskip("torch")
    from meep_gb300.design import DesignDFT, DesignProblem2D

    prob = DesignProblem2D(_lib.Engine(engine_lib), nx=120, ny=80, design=(20, 20), steps=800)
    rng = np.random.default_rng(7)
    eps_np = rng.uniform(1.0, 12.0, size=prob.design)
    eps = torch.tensor(eps_np, dtype=torch.float64, requires_grad=True)
    F = DesignDFT.apply(eps, prob, 0)
    J = (F.abs() ** 2).mean(0).sum()
    J.backward()
    F2, handle = prob.run(eps_np, grad=True, checkpoint_every=0)
    J2, dJdF = prob.objective(F2)
    g2 = prob.backward(handle, dJdF)
    assert abs(J.item() - J2) <= 1e-12 * abs(J2)
    assert relerr(eps.grad.numpy(), g2) <= 1e-12
