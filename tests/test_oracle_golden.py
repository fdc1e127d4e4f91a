"""CPU: pin the oracle (host code + CPU restatement, oracle/) against the
reference's own outputs (tests/golden, produced by the reference core built
from its sources) and its known-answer values (tests/known_results.cpp)."""
import pytest

from harness import ORACLE_DRIVER, compare_records, golden, relerr, run_driver

SMALL = ["tm2d_small", "tm2d_small_dec1", "vec3d_small", "disp3d_small"]


@pytest.mark.parametrize("case", SMALL + ["known"])
def test_oracle_fp64_matches_reference(case, oracle_lib, tmp_path):
    ref = golden(case, "f64")
    out = run_driver(ORACLE_DRIVER[64], case, tmp_path)
    if case == "known":
        for k, v in ref.items():
            assert out[k][0] == v[0], (k, out[k][0], v[0])
        return
    for k, err in compare_records(out, ref, case).items():
        # fields are bit-identical; DFT/flux differ only by summation order
        assert err <= 1e-13, (case, k, err)


def test_known_results_values(oracle_lib, tmp_path):
    # published values of the reference's test suite (tests/known_results.cpp:146-165),
    # including the Bloch-periodic ones
    out = run_driver(ORACLE_DRIVER[64], "known", tmp_path)
    expect = {"metallic_2d_tm": 5.20605, "pml_2d_tm": 0.883776, "metallic_3d": -41.8057,
              "polariton_1d": -0.0894851, "x_periodic_2d": 0.110425, "periodic_2d_rods": -4.78767,
              "periodic_2d": 1.12502, "x_periodic_y_pml_2d": 0.608815, "x_periodic_3d": -100.758,
              "x_periodic_y_pml_3d": -101.398, "periodic_3d_rods": -103.844, "periodic_3d": -99.1618}
    for k, v in expect.items():
        assert abs(out[k][0] - v) <= abs(v) * 1e-5, (k, out[k][0], v)


@pytest.mark.parametrize("case", ["tm2d_small", "vec3d_small", "disp3d_small"])
def test_oracle_fp32_close_to_reference_fp64(case, oracle_lib, tmp_path):
    """Single precision: no worse than 3x the reference's own FP32 build,
    measured against the reference FP64 build on the same case."""
    ref = golden(case, "f64")
    ref32 = compare_records(golden(case, "f32"), ref, case)
    out = compare_records(run_driver(ORACLE_DRIVER[32], case, tmp_path), ref, case)
    for k, err in out.items():
        assert err <= max(3 * ref32[k], 1e-6), (case, k, err, ref32[k])


def test_oracle_full_2d_flux(oracle_lib, tmp_path):
    """512x512 TM, 40 cylinders, 4000 steps, 51-frequency flux: same flux as
    the reference FP64 build to 1e-10."""
    ref = golden("tm2d_full", "f64")
    out = run_driver(ORACLE_DRIVER[64], "tm2d_full", tmp_path)
    assert relerr(out["flux"], ref["flux"]) <= 1e-10
