"""GPU: the CUDA engine behind the meep:: drop-in, driven by the same golden
driver source as the reference, against the reference's own outputs."""
import pytest

from harness import GPU_DRIVER, compare_records, golden, relerr, run_driver

pytestmark = pytest.mark.gpu

SMALL = ["tm2d_small", "tm2d_small_dec1", "vec3d_small", "disp3d_small"]


@pytest.mark.parametrize("case", SMALL)
def test_gpu_fp64_matches_reference(case, gpu_drivers, tmp_path):
    """FP64 GPU path vs the reference FP64 build: fields, DFT spectra and flux
    within 1e-10 relative (observed: bit-identical fields)."""
    ref = golden(case, "f64")
    out = run_driver(GPU_DRIVER[64], case, tmp_path)
    for k, err in compare_records(out, ref, case).items():
        assert err <= 1e-10, (case, k, err)


def test_gpu_known_results(gpu_drivers, tmp_path):
    ref = golden("known", "f64")
    out = run_driver(GPU_DRIVER[64], "known", tmp_path)
    for k, v in ref.items():
        assert relerr(out[k], v) <= 1e-10, (k, out[k], v)


@pytest.mark.parametrize("case", ["tm2d_small", "vec3d_small", "disp3d_small"])
def test_gpu_fp32_close_to_reference_fp64(case, gpu_drivers, tmp_path):
    """FP32 GPU path: no worse than 3x the reference's own FP32 build."""
    ref = golden(case, "f64")
    ref32 = compare_records(golden(case, "f32"), ref, case)
    out = compare_records(run_driver(GPU_DRIVER[32], case, tmp_path), ref, case)
    for k, err in out.items():
        assert err <= max(3 * ref32[k], 1e-6), (case, k, err, ref32[k])


def test_gpu_full_2d_flux(gpu_drivers, tmp_path):
    """512x512 TM, 4000 steps, 51 frequencies: flux within 1e-10 of the
    reference FP64 build; FP32 flux within 1e-5."""
    ref = golden("tm2d_full", "f64")
    out = run_driver(GPU_DRIVER[64], "tm2d_full", tmp_path)
    assert relerr(out["flux"], ref["flux"]) <= 1e-10
    out32 = run_driver(GPU_DRIVER[32], "tm2d_full", tmp_path)
    assert relerr(out32["flux"], ref["flux"]) <= 1e-5
