"""Subpixel averaging and off-diagonal inverse permittivity.

Cases of tests/golden/golden_driver.cpp run by the reference core (fixtures)
and by the meep:: drop-in over the oracle (CPU) or the CUDA engine (GPU):
  aniso1d        1-D slab with faces between grid points, averaged
  aniso_te2d     2-D TE, averaged disk + tilted slab, PML, Lorentzian in the
                 disk, D conductivity, integrated Ey and current Hz sources
  aniso3d        3-D sphere + slab with a normal along no axis (full 3x3
                 tensors), PML, Lorentzian, two integrated sources, flux
  offdiag_te2d   constant xy off-diagonal tensor everywhere incl. the PML
                 (the tensor of the reference's tests/pml.cpp), B conductivity
  aniso_bloch2d  averaged disk lattice with a Bloch wavevector (complex
                 fields; the off-diagonal terms read D and P on ghost planes)
Records: fields, flux, and the chi1inv tensor entries (structure::get_chi1inv)
at every Yee point."""
import os
import subprocess

import numpy as np
import pytest

from harness import GPU_DRIVER, ORACLE_DRIVER, compare_records, golden, run_driver

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASES = ["aniso1d", "aniso_te2d", "aniso3d", "offdiag_te2d", "aniso_bloch2d"]


def test_sphere_quadrature_matches_reference(tmp_path):
    """The quadrature table of the normal-vector estimate (McLaren's 50-point
    formula, 12 points on the circle, the two poles, greedily reordered) is
    bit-identical to the table the reference's generator prints."""
    src = tmp_path / "dump.cpp"
    src.write_text('#include <cstdio>\n#include "subpixel.hpp"\nint main() {\n'
                   '  const auto &q = mgb_subpixel::sphere_quadrature();\n'
                   '  for (int d = 0; d < 3; d++)\n    for (int i = 0; i < q.n[d]; i++)\n'
                   '      printf("%d %d %.17g %.17g %.17g %.17g\\n", d + 1, i, q.pt[d][i][0], q.pt[d][i][1],'
                   ' q.pt[d][i][2], q.pt[d][i][3]);\n}\n')
    exe = tmp_path / "dump"
    csrc = os.path.join(ROOT, "meep_gb300", "csrc")
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-I" + csrc, str(src),
                    os.path.join(csrc, "sphere_quadrature.cpp"), "-o", str(exe)], check=True)
    mine = [line.split() for line in subprocess.run([str(exe)], check=True, capture_output=True,
                                                    text=True).stdout.splitlines()]
    ref = [line.split() for line in open(os.path.join(ROOT, "tests", "golden", "sphere_quad.txt"))]
    assert len(mine) == len(ref) == 64
    for a, b in zip(mine, ref):
        assert a[:2] == b[:2]
        assert [float(v) for v in a[2:]] == [float(v) for v in b[2:]], (a, b)


def _check_fp64(out, ref, case):
    for k, err in compare_records(out, ref, case).items():
        if k == "flux":
            assert err <= 1e-13, (case, k, err)  # summation order only
        else:
            assert np.array_equal(np.asarray(out[k]), np.asarray(ref[k])), (case, k, err)


@pytest.mark.parametrize("case", CASES)
def test_oracle_fp64_matches_reference(case, oracle_lib, tmp_path):
    """Averaged tensors and fields bit-identical to the reference FP64 build."""
    _check_fp64(run_driver(ORACLE_DRIVER[64], case, tmp_path), golden(case, "f64"), case)


@pytest.mark.parametrize("case", ["aniso_te2d", "offdiag_te2d", "aniso_bloch2d"])
def test_oracle_fp32_close_to_reference_fp64(case, oracle_lib, tmp_path):
    """Single precision: no worse than 3x the reference's own FP32 build (whose
    OFFDIAG sums promote to double through the literal 0.25; here they stay in
    float, as on the GPU)."""
    ref = golden(case, "f64")
    ref32 = compare_records(golden(case, "f32"), ref, case)
    out = compare_records(run_driver(ORACLE_DRIVER[32], case, tmp_path), ref, case)
    for k, err in out.items():
        assert err <= max(3 * ref32[k], 1e-6), (case, k, err, ref32[k])


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_gpu_fp64_matches_reference(case, gpu_drivers, tmp_path):
    """The CUDA engine with off-diagonal tensors: bit-identical fields."""
    _check_fp64(run_driver(GPU_DRIVER[64], case, tmp_path), golden(case, "f64"), case)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["aniso_te2d", "aniso3d", "offdiag_te2d", "aniso_bloch2d"])
def test_gpu_fp32_close_to_reference_fp64(case, gpu_drivers, tmp_path):
    """FP32 fields no worse than 3x the reference's FP32 build; FP32 flux (the
    blocked DFT contraction, FP32 sums of 64 samples) within the 1e-5 flux
    tolerance of the FP32 engine."""
    ref = golden(case, "f64")
    ref32 = compare_records(golden(case, "f32"), ref, case)
    out = compare_records(run_driver(GPU_DRIVER[32], case, tmp_path), ref, case)
    for k, err in out.items():
        floor = 1e-5 if k == "flux" else 1e-6
        assert err <= max(3 * ref32[k], floor), (case, k, err, ref32[k])


def _random_geometry(rng, n):
    objs = []
    for _ in range(n):
        kind = int(rng.integers(0, 3))
        ax = rng.normal(size=3)
        ax /= np.linalg.norm(ax)
        objs.append({"kind": kind, "center": rng.uniform(-1, 1, 3), "size": rng.uniform(0.2, 1.2, 3),
                     "radius": rng.uniform(0.1, 0.6), "height": rng.uniform(0.3, 2.0), "axis": ax,
                     "eps": rng.uniform(1.5, 12.0)})
    return objs


def _pixels(rng, dim, n, res=10.0):
    k = rng.integers(-15, 16, size=(n, 3)) * 2 + rng.integers(0, 2, size=(n, 3))
    cen = k * (0.5 / res)
    if dim == 2:
        cen[:, 2] = 0
    if dim == 1:
        cen[:, :2] = 0
    lo, hi = cen - 0.5 / res, cen + 0.5 / res
    if dim == 2:
        lo[:, 2] = hi[:, 2] = 0
    if dim == 1:
        lo[:, :2] = hi[:, :2] = 0
    return lo, hi


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [1, 2, 3])
def test_device_rows_match_host(dim, engine_lib, oracle_lib):
    """mfd_subpixel_rows on the GPU equals the same routine on the host bit for
    bit, over random objects and pixels (many of them on interfaces)."""
    from meep_gb300 import _lib
    rng = np.random.default_rng(7 + dim)
    objs = _random_geometry(rng, 12)
    lo, hi = _pixels(rng, dim, 20000)
    for cdir in range(3):
        gpu = _lib.Engine(engine_lib).subpixel_rows(dim, cdir, lo, hi, objs, eps_default=1.3)
        cpu = _lib.Engine(oracle_lib).subpixel_rows(dim, cdir, lo, hi, objs, eps_default=1.3)
        if dim > 1 and cdir < 2:
            assert np.count_nonzero(cpu[:, 1 - cdir]) > 100  # interface pixels with off-diagonal entries
        assert np.array_equal(gpu, cpu), (dim, cdir, int(np.count_nonzero(gpu != cpu)))


def test_host_rows_cases(oracle_lib):
    """CPU: uniform pixels give 1/eps on the diagonal; an interface pixel of a
    plane x = 0 gives the harmonic/arithmetic means along/against the normal."""
    from meep_gb300 import _lib
    eng = _lib.Engine(oracle_lib)
    objs = [{"kind": 0, "center": (-5, 0, 0), "size": (10, 100, 100), "eps": 4.0}]
    lo = np.array([[1.0, 1.0, 1.0], [-0.05, -0.05, -0.05]])
    hi = lo + 0.1
    rx = eng.subpixel_rows(3, 0, lo, hi, objs)
    ry = eng.subpixel_rows(3, 1, lo, hi, objs)
    assert rx[0].tolist() == [1.0, 0.0, 0.0] and ry[0].tolist() == [0.0, 1.0, 0.0]
    # half-filled pixel: E normal to the interface sees <1/eps>, E along it 1/<eps>
    assert abs(rx[1, 0] - 0.5 * (1 + 0.25)) < 0.02
    assert abs(ry[1, 1] - 1 / 2.5) < 0.02
    assert abs(rx[1, 1]) < 1e-12 and abs(ry[1, 0]) < 1e-12
