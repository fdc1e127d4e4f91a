"""GPU: the reverse-time adjoint on 3-D full-vector problems with PML on every
face and a flux objective (E and H monitors): against central finite
differences in FP64, checkpointed against recorded, FP32 against FP64, and
the full-size design workload (192x192x128, 64x64x16 design voxels, 2000
steps, sqrt(T) checkpoints)."""
import numpy as np
import pytest

from harness import relerr
from meep_gb300 import _lib
from meep_gb300.design import DesignProblem3D

pytestmark = pytest.mark.gpu

SMALL = dict(n=(28, 28, 32), res=10.0, dpml_cells=4, slab=(10, 13), design=(4, 4, 3), plane_z=24, plane=12, src_z=6,
             fcen=0.25, df=0.1, nfreq=5, steps=300)


@pytest.fixture(scope="module")
def small(engine_lib):
    prob = DesignProblem3D(_lib.Engine(engine_lib), **SMALL)
    eps = np.random.default_rng(3).uniform(1.0, 12.0, size=SMALL["design"])
    return prob, eps


def _grad(prob, eps, precision, checkpoint_every):
    J, F, handle = prob.run(eps, grad=True, checkpoint_every=checkpoint_every, precision=precision)
    return J, prob.backward(handle, F)


def _fd(prob, eps, vox, h=1e-4):
    out = []
    for v in vox:
        ep = eps.copy()
        ep[v] += h
        em = eps.copy()
        em[v] -= h
        out.append((prob.run(ep, precision=64)[0] - prob.run(em, precision=64)[0]) / (2 * h))
    return np.array(out)


def test_adjoint3d_matches_finite_differences(small):
    prob, eps = small
    J, g = _grad(prob, eps, 64, 0)
    assert J != 0.0
    rng = np.random.default_rng(8)
    vox = [tuple(int(rng.integers(0, s)) for s in SMALL["design"]) for _ in range(6)]
    fd = _fd(prob, eps, vox)
    adj = np.array([g[v] for v in vox])
    assert relerr(adj, fd) <= 1e-6, (adj, fd)


def test_adjoint3d_bands_equal_per_component(small, monkeypatch):
    """The reversed steps on the 3-D band kernels give the gradient of the
    per-component adjoint kernels to the bit (same per-point arithmetic and
    gather order)."""
    prob, eps = small
    _, g_band = _grad(prob, eps, 64, 0)
    monkeypatch.setenv("MFD_GENERIC_KERNELS", "1")
    _, g_comp = _grad(prob, eps, 64, 0)
    assert np.array_equal(g_band, g_comp)


def test_adjoint3d_checkpointed_equals_recorded(small):
    prob, eps = small
    _, g_rec = _grad(prob, eps, 64, 0)
    _, g_ck = _grad(prob, eps, 64, 17)
    assert relerr(g_ck, g_rec) <= 1e-12


def test_adjoint3d_fp32_close_to_fp64(small):
    prob, eps = small
    _, g64 = _grad(prob, eps, 64, 0)
    _, g32 = _grad(prob, eps, 32, 0)
    assert relerr(g32, g64) <= 1e-3


def test_design3d_full_size_vs_fd(engine_lib):
    """192x192x128 cells at resolution 20, 16-cell PML, 64x64x16 design voxels
    (eps uniform in [1, 12] from a seed) on an eps = 2.1 slab, Ex dipole, flux
    through a 128x128 plane at 20 frequencies, 2000 steps.  Gradient in FP32
    fields / FP64 DFT sums with sqrt(T) checkpoints (every 45 steps) and in
    FP64, against central finite differences (h = 1e-4, FP64) at 10 voxels."""
    torch = pytest.importorskip("torch")
    prob = DesignProblem3D(_lib.Engine(engine_lib))
    rng = np.random.default_rng(2025)
    eps = rng.uniform(1.0, 12.0, size=prob.design_shape)
    free0 = torch.cuda.mem_get_info()[0]
    J32, F32, handle = prob.run(eps, grad=True, checkpoint_every=45, precision=32)
    free1 = torch.cuda.mem_get_info()[0]
    g32 = prob.backward(handle, F32)
    _, g64 = _grad(prob, eps, 64, 45)
    vox = [tuple(int(rng.integers(0, s)) for s in prob.design_shape) for _ in range(10)]
    fd = _fd(prob, eps, vox)
    e64 = relerr(np.array([g64[v] for v in vox]), fd)
    e32 = relerr(np.array([g32[v] for v in vox]), fd)
    print("3-D design: J=%.6g, FP64 adjoint vs FD %.2e, FP32 adjoint vs FD %.2e, forward state + checkpoints %.2f GB"
          % (J32, e64, e32, (free0 - free1) / 1e9))
    assert e64 <= 1e-4
    assert e32 <= 1e-3
    assert (free0 - free1) < 80e9
