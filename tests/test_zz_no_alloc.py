"""GPU: the allocation-free flux reduction (mfd_flux_noalloc) against the
engine's own flux (mfd_flux) and against a float64 numpy sum.

Collected last so that it runs both alone and after every other GPU test (the
scratch array it uses then holds whatever an earlier call left there)."""
import ctypes as C

import numpy as np
import pytest

from meep_gb300 import _lib

torch = pytest.importorskip("torch")


def _noalloc(eng, E, H):
    """Upload E, H ([npts, nfreq] complex128) and reduce them on the device."""
    npts, nf = E.shape
    dE = torch.from_numpy(np.ascontiguousarray(E)).view(torch.float64).cuda()
    dH = torch.from_numpy(np.ascontiguousarray(H)).view(torch.float64).cuda()
    out = torch.full((nf,), float("nan"), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = eng.lib.mfd_flux_noalloc(C.c_void_p(dE.data_ptr()), C.c_void_p(dH.data_ptr()), npts, nf,
                                  C.c_void_p(out.data_ptr()), C.c_void_p(stream))
    assert rc == 0, eng.lib.mfd_noalloc_last_error().decode()
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _flux_problem(eng):
    """3-D vacuum box with PML, an Ez point source and a 30x30 Ex/Hy flux
    plane (with 40 frequencies) normal to z."""
    n = (40, 40, 40)
    comps = [_lib.comp(t, d) for t in range(4) for d in range(3)]
    pml = {(d, s): (0.5, 1e-15, 1.0) for d in range(3) for s in (0, 1)}
    sim = _lib.Sim(eng, dim=3, n=n, io=(-40, -40, -40), a=10.0, courant=0.5, pml=pml, precision=64,
                   components=comps)
    ez = _lib.comp(_lib.E, _lib.Z)
    src = sim.add_gaussian_src(0.6, 0.4)
    sim.add_source_points(ez, src, [(20 * sim.ext[1] + 20) * sim.ext[2] + 16], [1.0])
    freqs = np.linspace(0.4, 0.8, 40)
    w = [np.ones(30), np.ones(30), np.ones(1)]
    lo, hi = (5, 5, 30), (34, 34, 30)
    mE = sim.add_dft(_lib.comp(_lib.E, _lib.X), lo, hi, w, dV=1.0, include_weights=False, scale=1.0,
                     centered=False, freqs=freqs, decimation=1)
    mH = sim.add_dft(_lib.comp(_lib.H, _lib.Y), lo, hi, w, dV=1.0, include_weights=False, scale=1.0,
                     centered=False, freqs=freqs, decimation=1)
    sim.step(80)
    return sim, mE, mH, len(freqs)


@pytest.mark.gpu
def test_noalloc_matches_engine_flux():
    eng = _lib.Engine()
    sim, mE, mH, nf = _flux_problem(eng)
    ref = sim.flux([mE], [mH], nf)
    E, H = sim.get_dft(mE), sim.get_dft(mH)
    sim.close()
    assert np.any(ref != 0.0)
    tol = 1e-12 * np.max(np.abs(ref))
    for _ in range(2):  # two calls in a row: the scratch keeps the first call's rows
        got = _noalloc(eng, E, H)
        assert np.max(np.abs(got - ref)) <= tol


@pytest.mark.gpu
def test_noalloc_large_and_small_in_turn():
    """More points than scratch rows (folded partial sums), then a small call
    that must not see the large call's leftover rows."""
    eng = _lib.Engine()
    rng = np.random.default_rng(11)
    for npts, nf in ((400_000, 24), (700, 1024), (3, 5), (400_000, 24)):
        E = rng.standard_normal((npts, nf)) + 1j * rng.standard_normal((npts, nf))
        H = rng.standard_normal((npts, nf)) + 1j * rng.standard_normal((npts, nf))
        ref = np.sum((E * np.conj(H)).real, axis=0)
        for _ in range(2):
            got = _noalloc(eng, E, H)
            assert np.allclose(got, ref, rtol=1e-12, atol=1e-12 * np.sqrt(npts))


@pytest.mark.gpu
def test_noalloc_rejects_oversize():
    eng = _lib.Engine()
    d = torch.zeros(2 * 2 * 2048, dtype=torch.float64, device="cuda")
    p = C.c_void_p(d.data_ptr())
    assert eng.lib.mfd_flux_noalloc(p, p, 2, 2048, p, None) != 0
    assert b"exceeds the scratch limit" in eng.lib.mfd_noalloc_last_error()
    assert eng.lib.mfd_flux_noalloc(p, p, 0, 4, p, None) != 0
