"""Shared helpers for the tests: run the golden driver builds, compare records,
and build seeded random problems for the C ABI."""
import os
import subprocess

import numpy as np

from meep_gb300 import _lib
from records import read_records

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
ORACLE_DRIVER = {64: os.path.join(ROOT, "oracle", "_build", "golden_driver64"),
                 32: os.path.join(ROOT, "oracle", "_build", "golden_driver32")}
GPU_DRIVER = {64: os.path.join(ROOT, "meep_gb300", "lib", "golden_driver64"),
              32: os.path.join(ROOT, "meep_gb300", "lib", "golden_driver32")}


def golden(case, prec="f64"):
    return read_records(os.path.join(GOLDEN, "%s.%s.bin" % (case, prec)))


def run_driver(exe, case, tmpdir, steps=None, threads=8):
    out = os.path.join(str(tmpdir), "%s.%s.bin" % (case, os.path.basename(exe)))
    cmd = [exe, case, out] + ([str(steps)] if steps else [])
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    subprocess.run(cmd, check=True, env=env, timeout=1800)
    return read_records(out)


def relerr(a, b):
    """max |a - b| / max |b| (infinity-norm relative error, as the reference's
    ApproxComparisonTestCase.assertClose does, python/tests/utils.py:10-29).
    Complex inputs are compared as complex numbers (|a - b| is the modulus
    of the difference), so the imaginary parts count."""
    a = np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape, (a.shape, b.shape)
    if np.iscomplexobj(a) or np.iscomplexobj(b):
        a = a.astype(np.complex128)
        b = b.astype(np.complex128)
    else:
        a = a.astype(np.float64)
        b = b.astype(np.float64)
    if a.size == 0:
        return 0.0
    m = np.abs(b).max()
    return float(np.abs(a - b).max() / m) if m > 0 else float(np.abs(a - b).max())


DFT_LAYOUT = {"tm2d_small": (2, 11), "tm2d_small_dec1": (2, 11), "vec3d_small": (3, 9),
              "disp3d_small": (3, 7)}


def split_dft(rec, case):
    """A dft_* record holds, per point, its ivec coordinates then (re, im) per
    frequency; return (coords, complex values[npts, nfreq])."""
    dim, nf = DFT_LAYOUT[case]
    arr = np.asarray(rec).reshape(-1, dim + 2 * nf)
    return arr[:, :dim], arr[:, dim::2] + 1j * arr[:, dim + 1::2]


def compare_records(out, ref, case, skip=("t", "realnum_bytes")):
    """Per-record relative errors, DFT records split into coordinates (must be
    equal) and values."""
    errs = {}
    for k, v in ref.items():
        if k in skip:
            continue
        assert k in out, k
        if k.startswith("dft_"):
            c0, v0 = split_dft(v, case)
            c1, v1 = split_dft(out[k], case)
            assert np.array_equal(c0, c1), (case, k, "coordinates differ")
            m = np.abs(v0).max()
            errs[k] = float(np.abs(v1 - v0).max() / m) if m else float(np.abs(v1 - v0).max())
        else:
            errs[k] = relerr(out[k], v)
    return errs


def random_problem(sim_factory, seed, dim, precision=64, poles=True, cond=True, pml=True,
                   nsrc=3, steps=60, n=None, bloch=None, bloch_pml=False, offdiag=False, ecur=True,
                   boxed=False, palette=False, bcond=False, poles_below=None, hcur=True, hmon=True,
                   src_box=None, decimation=2):
    """Build the same seeded random problem on one engine and return outputs.

    Random inverse permittivities, conductivities and Lorentz/Drude sigma
    arrays on a small grid with PML; integrated E sources at random points and
    a current source; two DFT monitors.  Returns dict of field arrays and DFT
    sums after `steps` steps; `n` overrides the random grid size.  offdiag:
    off-diagonal inverse permittivities on 40% of the points (Ex: xy and xz,
    Ey: yz only, Ez: zy only -- the reference's 3x3, 2x2 and swapped 2x2
    cases); ecur=False makes every E source integrated (no D current).
    boxed: conductivities and pole strengths are zero outside random boxes
    (separate ones per array), so long grids hold runs of points where a
    pole or a conductivity is absent next to runs where it is present.
    palette: permittivities, conductivities and pole strengths take a few
    values only (eps 1, 4, 12; conductivity 0, 0.3; sigma 0, 0.7, 1.5), as
    in structures built from a few media.
    bcond: conductivities on the B components too.
    poles_below: pole strengths zero at z points >= poles_below (a layer of
    dispersive medium at the low z end, as the dispersive benchmark has).
    hcur=False: no H current source; hmon=False: the second monitor on a D
    component instead of H (no flux); src_box=(lo, hi): E source points only
    inside that index box (inclusive); decimation: of both monitors."""
    rng = np.random.default_rng(seed)
    nrand = n
    if dim == 2:
        n = (int(rng.integers(28, 40)), int(rng.integers(24, 36)), 0)
        comps = [_lib.comp(_lib.E, _lib.Z), _lib.comp(_lib.D, _lib.Z), _lib.comp(_lib.H, _lib.X),
                 _lib.comp(_lib.B, _lib.X), _lib.comp(_lib.H, _lib.Y), _lib.comp(_lib.B, _lib.Y)]
    else:
        n = (int(rng.integers(18, 24)), int(rng.integers(16, 22)), int(rng.integers(14, 20)))
        comps = [_lib.comp(t, d) for t in range(4) for d in range(3)]
    if nrand is not None:
        n = tuple(nrand)
    io = [-(n[d] - n[d] % 2) for d in range(3)]
    a = 10.0
    pmlspec = {}
    if pml:
        for d in range(dim if dim == 3 else 2):
            for side in (0, 1):
                pmlspec[(d, side)] = (float(rng.choice([0.3, 0.5])), 1e-15, 1.0)
                if bloch is not None and d in bloch and not bloch_pml:
                    del pmlspec[(d, side)]  # periodic direction without PML
    sim = sim_factory(dim=dim, n=n, io=io, a=a, courant=0.5, pml=pmlspec, precision=precision,
                      components=comps)
    if bloch is not None:
        sim.set_bloch([int(d in bloch) for d in range(3)], [bloch.get(d, 0.0) for d in range(3)])
    ext = sim.ext
    shape = tuple(ext)
    def pal(arr, values):
        """the palette value nearest to each entry"""
        v = np.asarray(values)
        return v[np.abs(np.asarray(arr)[..., None] - v).argmin(axis=-1)]

    for c in comps:
        if c // 3 == _lib.E:
            eps = rng.uniform(1.0, 12.0, size=shape)
            sim.set_chi1inv(c, c % 3, 1.0 / (pal(eps, [1.0, 4.0, 12.0]) if palette else eps))
    if offdiag:
        for c, dirs in ((_lib.comp(_lib.E, 0), (1, 2)), (_lib.comp(_lib.E, 1), (2,)), (_lib.comp(_lib.E, 2), (1,))):
            if c not in comps:
                continue
            for d in dirs:
                arr = np.where(rng.uniform(size=shape) < 0.4, rng.uniform(-0.08, 0.08, size=shape), 0.0)
                sim.set_chi1inv(c, d, arr)
    def box_mask():
        m = np.zeros(shape, dtype=bool)
        lo = [int(rng.integers(0, max(1, e // 2))) for e in shape]
        hi = [lo[d] + int(rng.integers(1, shape[d] - lo[d] + 1)) for d in range(3)]
        m[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]] = True
        return m

    if cond:
        for c in comps:
            if c // 3 == _lib.D or (bcond and c // 3 == _lib.B):
                arr = np.where(rng.uniform(size=shape) < 0.3, rng.uniform(0, 0.5, size=shape), 0.0)
                if boxed:
                    arr = np.where(box_mask(), rng.uniform(0, 0.5, size=shape), 0.0)
                if palette:
                    arr = pal(arr, [0.0, 0.3])
                sim.set_conductivity(c, arr)
    if poles:
        for (w0, g, dr) in ((1e-5, 0.05, True), (0.8, 0.1, False)):
            sig = []
            for d in range(3):
                c = _lib.comp(_lib.E, d)
                arr = rng.uniform(0, 2.0, size=shape) if c in comps else None
                if boxed and arr is not None:
                    arr = np.where(box_mask(), arr, 0.0)
                if poles_below is not None and arr is not None:
                    # poles only in the low z layer (points k_z < poles_below)
                    arr = arr.copy()
                    arr[..., poles_below:] = 0.0
                if palette and arr is not None:
                    arr = pal(arr, [0.0, 0.7, 1.5])
                sig.append(arr)
            sim.add_lorentzian(w0, g, dr, sig)
    ecomps = [c for c in comps if c // 3 == _lib.E]
    s_int = sim.add_gaussian_src(0.6, 2.0, integrated=True)
    s_cur = sim.add_gaussian_src(0.5, 1.5, integrated=False)
    ndense = int(np.prod(shape))
    pool = np.arange(ndense)
    if src_box is not None:
        kk = np.indices(shape).reshape(len(shape), -1)
        inside = np.ones(ndense, dtype=bool)
        for d in range(len(shape)):
            inside &= (kk[d] >= src_box[0][d]) & (kk[d] <= src_box[1][d])
        pool = pool[inside]
    for j in range(nsrc):
        c = ecomps[j % len(ecomps)]
        idx = rng.choice(pool, size=4, replace=False)
        amp = rng.normal(size=4) + 1j * rng.normal(size=4)
        sim.add_source_points(c, s_int if (j or not ecur) else s_cur, idx, amp)
    # an H current source
    hc = [c for c in comps if c // 3 == _lib.H][0]
    hidx = rng.choice(ndense, size=3, replace=False)
    hamp = rng.normal(size=3)
    if hcur:
        sim.add_source_points(hc, s_cur, hidx, hamp)
    mons = []
    second = [c for c in comps if c // 3 == (_lib.H if hmon else _lib.D)][-1]
    for c in (ecomps[0], second):
        lo = [1 if ext[d] > 1 else 0 for d in range(3)]
        hi = [ext[d] - 3 if ext[d] > 1 else 0 for d in range(3)]
        w = [rng.uniform(0.2, 1.0, size=hi[d] - lo[d] + 1) if ext[d] > 1 else None for d in range(3)]
        mons.append(sim.add_dft(c, lo, hi, w, dV=0.01, include_weights=True, scale=0.3 - 0.2j,
                                centered=True, freqs=np.linspace(0.3, 0.9, 5), decimation=decimation))
    sim.step(steps)
    out = {"c%d" % c: sim.get_field(c) for c in comps}
    if bloch is not None:
        out.update({"i%d" % c: sim.get_field_im(c) for c in comps})
    for m in mons:
        out["dft%d" % m] = sim.get_dft(m)
    if hmon:
        out["flux"] = sim.flux([mons[0]], [mons[1]], 5)
    sim.close()
    return out


# ---------------------------------------------------------------- adjoint
def tm2d_design_problem(eng, eps_design, precision=64, steps=600, checkpoint_every=0, grad=True,
                        nfreq=5, seed=3):
    """2-D TM problem for gradient tests: 72x56 cells, resolution 10, PML 0.5
    on all sides, eps=12 guide along x, an eps design block (given) in the
    middle, Gaussian Ez line source on the left, objective
    J = sum_w mean_k |DFT Ez(k, w)|^2 over a 9-point line on the right.
    Returns (J, dJ/deps over the design block or None)."""
    rng = np.random.default_rng(seed)
    n = (72, 56, 0)
    io = (-72, -56, 0)
    comps = [_lib.comp(_lib.E, _lib.Z), _lib.comp(_lib.D, _lib.Z), _lib.comp(_lib.H, _lib.X),
             _lib.comp(_lib.B, _lib.X), _lib.comp(_lib.H, _lib.Y), _lib.comp(_lib.B, _lib.Y)]
    pml = {(d, s): (0.5, 1e-15, 1.0) for d in (0, 1) for s in (0, 1)}
    sim = _lib.Sim(eng, dim=2, n=n, io=io, a=10.0, courant=0.5, pml=pml, precision=precision,
                   components=comps)
    ext = sim.ext
    eps = np.ones((ext[0], ext[1]))
    eps[:, 24:32] = 12.0                                  # guide
    eps += 0.2 * rng.uniform(size=eps.shape)              # weak background texture
    eps_design = np.asarray(eps_design, dtype=np.float64)
    lo = (28, 20, 0)
    hi = (lo[0] + eps_design.shape[0] - 1, lo[1] + eps_design.shape[1] - 1, 0)
    eps[lo[0]:hi[0] + 1, lo[1]:hi[1] + 1] = eps_design
    ez = _lib.comp(_lib.E, _lib.Z)
    sim.set_chi1inv(ez, _lib.Z, 1.0 / eps)
    src = sim.add_gaussian_src(0.35, 0.2)
    idx = [14 * ext[1] + j for j in range(24, 33)]
    sim.add_source_points(ez, src, idx, np.ones(len(idx)) * 10.0)
    line_lo, line_hi = (56, 24, 0), (56, 32, 0)
    w = [np.ones(1), np.ones(9), None]
    freqs = np.linspace(0.3, 0.4, nfreq)
    mid = sim.add_dft(ez, line_lo, line_hi, w, dV=1.0, include_weights=False, scale=1.0, centered=False,
                      freqs=freqs, decimation=1)
    if grad:
        sim.design([ez], lo, hi)
        sim.forward(steps, checkpoint_every)
    else:
        sim.step(steps)
    F = sim.get_dft(mid)                                   # [npts, nfreq]
    J = float(np.sum(np.abs(F) ** 2) / F.shape[0])
    g = None
    if grad:
        G = 2.0 * F / F.shape[0]                           # dJ/dRe F + i dJ/dIm F
        gchi = sim.backward({mid: G})[0, :, :, 0]
        chi = 1.0 / eps_design
        g = -gchi * chi * chi                              # chi = 1/eps
    sim.close()
    return J, g
